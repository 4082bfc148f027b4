// kinfu_run: the headless frame loop of the reference's system_interface.cpp:3-71 on
// kinfu_gb300, through the C++ KinfuPipeline of kinfu_pipeline.hpp.  The viewer and the
// OpenCV windows are not on this path: each frame prints the camera position as the
// reference's IncomingFrameProcessing does (kinfu_pipeline.cpp:164-167), and the loop
// can write the poses and the latest predicted surface out.
//
//   kinfu_run [--data DIR] [--start N] [--end N] [--every N]
//             [--precision] [--poses FILE] [--ply FILE] [--quiet]
//
// --data     directory of dep%04d.dat frames (../data as in the reference)
// --start, --end, --every   start_frame, end_frame, per_nth_frame (25, 300, 1)
// --precision   the precision form (FP16 TSDF, compensated sums, FP64 solve)
// --poses    write every frame's pose as 16 float32 (row-major) to FILE
// --ply      write the last frame's predicted surface as a binary PLY
// --quiet    print only the summary line
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kinfu_pipeline.hpp"

namespace {

struct Options {
    std::string data = "../data";
    int start = 25, end = 300, every = 1;
    bool precision = false, quiet = false;
    std::string poses, ply;
};

bool parse(int argc, char** argv, Options& o)
{
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&](const char* name) -> const char* {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "%s needs a value\n", name);
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "--data") o.data = next("--data");
        else if (a == "--start") o.start = std::atoi(next("--start"));
        else if (a == "--end") o.end = std::atoi(next("--end"));
        else if (a == "--every") o.every = std::atoi(next("--every"));
        else if (a == "--poses") o.poses = next("--poses");
        else if (a == "--ply") o.ply = next("--ply");
        else if (a == "--precision") o.precision = true;
        else if (a == "--quiet") o.quiet = true;
        else {
            std::fprintf(stderr, "unknown option %s\n", a.c_str());
            return false;
        }
    }
    return o.every > 0 && o.end >= o.start;
}

}  // namespace

int main(int argc, char** argv)
{
    Options o;
    if (!parse(argc, argv, o)) {
        std::fprintf(stderr, "usage: kinfu_run [--data DIR] [--start N] [--end N] [--every N] [--precision] "
                             "[--poses FILE] [--ply FILE] [--quiet]\n");
        return 2;
    }
    // image size and depth thresholds of system_interface.cpp:6-11
    const int height = 480, width = 640;
    const float max_depth = 2000.f, min_depth = 300.f;
    try {
        kf_config cfg = Kinfu::KinfuPipeline::default_config(height, width, max_depth, min_depth);
        if (o.precision) {
            cfg.tsdf_storage = KF_TSDF_F16;
            cfg.solve_mode = KF_SOLVE_PRECISE;
            cfg.icp_reduction = KF_REDUCE_TREE;
        }
        Kinfu::KinfuPipeline kinfu(cfg);
        kinfu.system_utility->SetDataDir(o.data);
        kinfu.copy_outputs = false;  // the viewer's planes are read once, at the end
        std::vector<float> poses;
        auto keep = [&]() { poses.insert(poses.end(), kinfu.extrinsic_matrix.begin(), kinfu.extrinsic_matrix.end()); };

        const auto t0 = std::chrono::steady_clock::now();
        kinfu.InitialProcessing(o.start);
        keep();
        int frames = 0;
        for (int f = o.start + o.every; f <= o.end; f += o.every) {
            kinfu.IncomingFrameProcessing(f, o.every);
            keep();
            ++frames;
            if (!o.quiet)
                std::printf("frame %d cam_pos %.4f %.4f %.4f\n", f, kinfu.extrinsic_matrix[3],
                            kinfu.extrinsic_matrix[7], kinfu.extrinsic_matrix[11]);
        }
        const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf("%d incoming frames + 1 initial in %.3f s: %.1f frames/s (frame files read, host buffers)\n",
                    frames, s, (frames + 1) / s);

        if (!o.poses.empty()) {
            FILE* fp = std::fopen(o.poses.c_str(), "wb");
            if (!fp || std::fwrite(poses.data(), sizeof(float), poses.size(), fp) != poses.size()) {
                std::fprintf(stderr, "cannot write %s\n", o.poses.c_str());
                if (fp) std::fclose(fp);
                return 1;
            }
            std::fclose(fp);
        }
        if (!o.ply.empty()) {
            int n = 0;
            Kinfu::check(kinfu.handle(), kf_export_ply(kinfu.handle(), o.ply.c_str(), nullptr, &n), "kf_export_ply");
            std::printf("%d predicted points written to %s\n", n, o.ply.c_str());
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "kinfu_run: %s\n", e.what());
        return 1;
    }
    return 0;
}
