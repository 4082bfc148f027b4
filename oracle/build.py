"""Build recipe for the CPU oracle (test infrastructure; never part of the product).

Two shared libraries, both compiled with ``-ffp-contract=off`` so that every float
operation rounds where the source expression says (gcc on aarch64 would otherwise
contract a*b+c into an FMA):

* ``oracle/libkf_oracle.so`` -- the restatement in ``kf_oracle.cpp`` and the FP64
  oracle in ``kf_oracle64.cpp``.
* ``oracle/_ref/libkf_ref.so`` -- the reference's own kernel bodies.  When the
  reference tree is available (its location in ``KF_REF_DIR``; no default) this
  splices the kernel bodies out of its ``src/parallel_processing`` sources into
  ``oracle/_ref/ref_kernels.inc`` (never committed: ``oracle/_ref/`` is git-ignored)
  and compiles them with ``ref_harness.cpp``.  Where the tree is absent but an
  earlier splice travelled with the checkout, that splice is compiled as is.

The splice keeps the reference text unchanged except for two substitutions, each
required to match exactly once:

1. ``int XY, XZ, YX, YZ, ZX, ZY;`` (voxel_traversal.cu:136) is zero-initialised.
   The reference reads these before assigning them when a ray reaches a zero
   crossing without having stepped along some axis; zero pins that case to "no hit",
   which is what g++ -O2 produces for the unmodified source.
2. After ``dev_surface_points_x[x] = surface_prediction.x;`` (voxel_traversal.cu:371)
   a ``KF_REF_HIT(x, voxel_index);`` hook records the zero-crossing voxel index, an
   output the reference computes but does not return.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_OUT = HERE / "_ref"
ORACLE_SO = HERE / "libkf_oracle.so"
REF_SO = REF_OUT / "libkf_ref.so"
REF_INC = REF_OUT / "ref_kernels.inc"

CXXFLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]

# (file, stop marker): everything before the first line starting with the marker,
# #include lines dropped
_SPLICE = [
    ("cuda_functions.cuh", None),
    ("projective_tsdf.cu", 'extern "C"'),
    ("raw_vertices.cu", 'extern "C"'),
    ("voxel_traversal.cu", 'extern "C"'),
    ("sensor_pose_estimation.cu", "void Cholesky_Decomposition"),
    ("bilateral_filtering.cu", 'extern "C"'),
]

_SUBST = {
    "voxel_traversal.cu": [
        ("int XY, XZ, YX, YZ, ZX, ZY;", "int XY = 0, XZ = 0, YX = 0, YZ = 0, ZX = 0, ZY = 0;"),
        ("dev_surface_points_x[x] = surface_prediction.x;",
         "dev_surface_points_x[x] = surface_prediction.x; KF_REF_HIT(x, voxel_index);"),
    ],
}


def reference_dir() -> Path | None:
    """The reference checkout named by KF_REF_DIR, or None (no splice is made)."""
    ref = os.environ.get("KF_REF_DIR")
    return Path(ref) if ref else None


def _newer(target: Path, sources) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(Path(s).stat().st_mtime <= t for s in sources)


def splice_reference(ref_dir: Path | None = None) -> Path | None:
    """Write oracle/_ref/ref_kernels.inc from the reference sources; None if absent."""
    ref_dir = ref_dir or reference_dir()
    if ref_dir is None:
        return None
    src_dir = ref_dir / "src" / "parallel_processing"
    if not src_dir.is_dir():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = ["/* generated by oracle/build.py from the reference sources -- do not commit */\n"]
    for name, stop in _SPLICE:
        path = src_dir / name
        lines = path.read_text().splitlines(keepends=True)
        body = []
        for n, line in enumerate(lines, start=1):
            if stop is not None and line.startswith(stop):
                break
            if line.lstrip().startswith("#include"):
                body.append("\n")
                continue
            body.append(line)
        text = "".join(body)
        for old, new in _SUBST.get(name, []):
            count = text.count(old)
            if count != 1:
                raise RuntimeError(f"{name}: expected exactly one '{old}', found {count}")
            text = text.replace(old, new)
        out.append(f'#line 1 "{path}"\n')
        out.append(text)
        out.append("\n")
    new_text = "".join(out)
    if not REF_INC.exists() or REF_INC.read_text() != new_text:
        REF_INC.write_text(new_text)
    return REF_INC


def _compile(out: Path, sources, extra=()) -> None:
    cmd = ["g++", *CXXFLAGS, *extra, "-o", str(out), *[str(s) for s in sources]]
    subprocess.run(cmd, check=True)


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / "kf_oracle.cpp", HERE / "kf_oracle64.cpp"]
    deps = srcs + [HERE / "kf_oracle.h", HERE / "ocv_restated.h"]
    if force or not _newer(ORACLE_SO, deps):
        _compile(ORACLE_SO, srcs)
    return ORACLE_SO


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference harness; None when no spliced reference is available."""
    splice_reference()
    if not REF_INC.exists():
        return None
    srcs = [HERE / "ref_harness.cpp"]
    deps = srcs + [REF_INC, HERE / "ref_shim.h", HERE / "kf_oracle.h", HERE / "ocv_restated.h"]
    if force or not _newer(REF_SO, deps):
        _compile(REF_SO, srcs, extra=["-I", str(HERE), "-Wno-unused-parameter", "-w"])
    return REF_SO


def build(force: bool = False) -> dict:
    return {"oracle": build_oracle(force), "ref": build_ref(force)}


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
