// C++ host side of kinfu_gb300: the reference's KinfuPipeline and SystemUtility
// interface (src/kinfu_pipeline.h:10-62, src/system_utility.h:11-65) over the C ABI of
// kinfu_gb300.h, without OpenCV.  A maintainer swaps the reference's headers for this one
// and keeps the calling code: the constructor's (height, width, max_depth, min_depth),
// InitialProcessing(start_frame) / IncomingFrameProcessing(current_frame, per_nth_frame)
// reading ../data/dep%04d.dat, extrinsic_matrix as the pose, and
// system_utility->ray_casting_data->surface_prediction_* as the predicted surface.
//
// What changes for the caller:
//   * cv::Mat members become Plane (row-major H x W floats) and std::array (the 3x3 and
//     4x4 matrices, row-major); the voxel arrays stay on the GPU (GetVolume copies them
//     out in the reference's z-fastest order on request);
//   * errors throw std::runtime_error with the library's message (the reference
//     ignores them);
//   * colour images (img%04d.jpg) are not loaded: the viewer is not on this path.
//
// Header-only; link with -lkinfu_gb300.
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "kinfu_gb300.h"

namespace Kinfu
{

// An image-sized float plane, row-major (the cv::Mat CV_32F stand-in).
struct Plane {
    int rows = 0, cols = 0;
    std::vector<float> data;

    Plane() = default;
    Plane(int r, int c) : rows(r), cols(c), data((size_t)r * c, 0.f) {}
    float* ptr(int r) { return data.data() + (size_t)r * cols; }
    const float* ptr(int r) const { return data.data() + (size_t)r * cols; }
    float& at(int r, int c) { return data[(size_t)r * cols + c]; }
    float at(int r, int c) const { return data[(size_t)r * cols + c]; }
};

// throws std::runtime_error for a failed call: the handle's message, or the status's
// name where there is no handle yet
inline void check(kf_handle* h, kf_status s, const char* what)
{
    if (s != KF_OK) throw std::runtime_error(std::string(what) + ": " + (h ? kf_last_error(h) : kf_status_string(s)));
}

// system_utility.h:11-65: image sizes, depth loading and the planes the viewer reads.
class SystemUtility
{
public:
    SystemUtility(int height, int width, float max_depth, float min_depth, std::string data_dir = "../data")
        : ray_casting_data(std::make_unique<RayCastingData>(height, width)),
          depth_data(std::make_unique<DepthImage3dData>(height, width)),
          initial_depth_image(height, width),
          _height(height),
          _width(width),
          _max_depth(max_depth),
          _min_depth(min_depth),
          _data_dir(std::move(data_dir))
    {
    }

    // LoadDepthData (system_utility.cpp:58-68): uint16 millimetres of data_dir/dep%04d.dat
    void LoadDepthData(std::vector<uint16_t>& depth_image, int frame_index) const
    {
        depth_image.resize((size_t)_height * _width);
        const kf_status s = kf_load_depth_dat(_data_dir.c_str(), frame_index, _height, _width, depth_image.data());
        if (s != KF_OK)
            throw std::runtime_error("cannot read " + _data_dir + "/dep" + std::to_string(frame_index) + ".dat");
    }

    struct RayCastingData {
        explicit RayCastingData(int h, int w)
            : surface_prediction_x(h, w),
              surface_prediction_y(h, w),
              surface_prediction_z(h, w),
              surface_prediction_normal_x(h, w),
              surface_prediction_normal_y(h, w),
              surface_prediction_normal_z(h, w)
        {
        }
        Plane surface_prediction_x, surface_prediction_y, surface_prediction_z;
        Plane surface_prediction_normal_x, surface_prediction_normal_y, surface_prediction_normal_z;
    };

    struct DepthImage3dData {
        explicit DepthImage3dData(int h, int w) : depth_image_next(h, w) {}
        Plane depth_image_next;  // the range-filtered depth of the latest incoming frame (mm)
    };

    std::unique_ptr<RayCastingData> ray_casting_data;
    std::unique_ptr<DepthImage3dData> depth_data;
    Plane initial_depth_image;  // the range-filtered depth of the first frame (mm)

    int GetImageHeight() const { return _height; }
    int GetImageWidth() const { return _width; }
    float GetMaxDepth() const { return _max_depth; }
    float GetMinDepth() const { return _min_depth; }
    const std::string& GetDataDir() const { return _data_dir; }
    void SetDataDir(std::string dir) { _data_dir = std::move(dir); }

private:
    int _height{0};
    int _width{0};
    float _max_depth{0.f};
    float _min_depth{0.f};
    std::string _data_dir;
};

// kinfu_pipeline.h:10-62: the frame loop.  The GPU volume, images and pose stay on the
// device between frames; after each frame call the pose is copied into extrinsic_matrix,
// and (with copy_outputs, the default) the predicted surface and the frame's filtered
// depth into system_utility, where the reference's viewer reads them.
class KinfuPipeline
{
public:
    // kinfu_pipeline.cpp:6-65: the reference's grid (360x360x300 at 10 mm from
    // (-2000, -2000, -1200) mm), truncation (300 / -30 / 300 mm) and intrinsics
    KinfuPipeline(int height, int width, float max_depth, float min_depth)
        : KinfuPipeline(default_config(height, width, max_depth, min_depth))
    {
    }

    // any kf_config (grid, ICP schedule, the precision form's storage and solve)
    explicit KinfuPipeline(const kf_config& cfg)
        : system_utility(std::make_unique<SystemUtility>(cfg.height, cfg.width, cfg.max_depth, cfg.min_depth))
    {
        check(nullptr, kf_create(&cfg, &_h), "kf_create");
        check(_h, kf_get_intrinsics(_h, intrinsic_matrix.data()), "kf_get_intrinsics");
        check(_h, kf_get_pose(_h, extrinsic_matrix.data()), "kf_get_pose");
    }

    ~KinfuPipeline()
    {
        if (_h) kf_destroy(_h);
    }
    KinfuPipeline(const KinfuPipeline&) = delete;
    KinfuPipeline& operator=(const KinfuPipeline&) = delete;

    // intrinsic_matrix: 3x3 row-major, 1-based principal point (kinfu_pipeline.cpp:14-24)
    std::array<float, 9> intrinsic_matrix{};
    // extrinsic_matrix: 4x4 row-major camera-to-world pose, mm
    std::array<float, 16> extrinsic_matrix{};
    std::unique_ptr<SystemUtility> system_utility;
    bool copy_outputs = true;

    // InitialProcessing (kinfu_pipeline.cpp:91-119): dep<start_frame>.dat
    void InitialProcessing(int start_frame)
    {
        system_utility->LoadDepthData(_frame, start_frame);
        InitialProcessing(_frame.data());
    }

    // IncomingFrameProcessing (kinfu_pipeline.cpp:121-193): dep<current_frame>.dat;
    // per_nth_frame is the caller's frame step, unused here as in the reference
    void IncomingFrameProcessing(int current_frame, int /*per_nth_frame*/)
    {
        system_utility->LoadDepthData(_frame, current_frame);
        IncomingFrameProcessing(_frame.data());
    }

    // the same on a depth image the caller holds (H*W uint16 mm, host memory)
    void InitialProcessing(const uint16_t* depth)
    {
        check(_h, kf_initial_processing(_h, depth), "kf_initial_processing");
        update(system_utility->initial_depth_image);
    }
    void IncomingFrameProcessing(const uint16_t* depth)
    {
        check(_h, kf_incoming_frame(_h, depth), "kf_incoming_frame");
        update(system_utility->depth_data->depth_image_next);
    }

    // the pose for the next frame (writes extrinsic_matrix through to the device)
    void SetPose(const std::array<float, 16>& T)
    {
        check(_h, kf_set_pose(_h, T.data()), "kf_set_pose");
        extrinsic_matrix = T;
    }

    // global_tsdf / global_weight_tsdf (kinfu_pipeline.h:23-24) in the reference's
    // z-fastest order, NaN where unobserved
    void GetVolume(std::vector<float>& tsdf, std::vector<float>& weight)
    {
        kf_config c;
        check(_h, kf_get_config(_h, &c), "kf_get_config");
        const size_t n = (size_t)c.dims[0] * c.dims[1] * c.dims[2];
        tsdf.resize(n);
        weight.resize(n);
        check(_h, kf_get_volume(_h, tsdf.data(), weight.data()), "kf_get_volume");
    }

    kf_handle* handle() const { return _h; }

    static kf_config default_config(int height, int width, float max_depth, float min_depth)
    {
        kf_config c;
        kf_config_default(&c);
        c.height = height;
        c.width = width;
        c.max_depth = max_depth;
        c.min_depth = min_depth;
        return c;
    }

private:
    void update(Plane& depth_out)
    {
        check(_h, kf_get_pose(_h, extrinsic_matrix.data()), "kf_get_pose");
        if (!copy_outputs) return;
        auto& r = *system_utility->ray_casting_data;
        check(_h,
              kf_get_predicted(_h, r.surface_prediction_x.data.data(), r.surface_prediction_y.data.data(),
                               r.surface_prediction_z.data.data(), r.surface_prediction_normal_x.data.data(),
                               r.surface_prediction_normal_y.data.data(), r.surface_prediction_normal_z.data.data()),
              "kf_get_predicted");
        check(_h, kf_get_depth(_h, depth_out.data.data()), "kf_get_depth");
    }

    kf_handle* _h = nullptr;
    std::vector<uint16_t> _frame;
};

}  // namespace Kinfu
