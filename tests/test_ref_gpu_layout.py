"""The ctypes restatements in oracle/ref_gpu.py of the reference's by-value
kernel parameter structs must have the reference's layout, field for field:
the reference cubins read them that way.  Checked where the reference tree and
nvcc are present (this test compiles static_asserts against the reference's
own headers; no GPU): sizes and every named member's offset."""
import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from oracle import ref_gpu

ROOT = Path(__file__).resolve().parents[1]
REF = Path(os.environ.get("SPH_REFERENCE_DIR", "/root/reference"))
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"

# (ctypes class, C++ type, members to check: ctypes name -> C++ member)
STRUCTS = [
    (ref_gpu.ParticleGPU, "particle_gpu", None),
    (ref_gpu.SegmentFEMGPU, "segment_FEM_gpu", None),
    (ref_gpu.IniState, "inistate_struct", None),
    (ref_gpu.DeviceBuffer, "grid_gpu_green::device_buffer", None),
    (ref_gpu.GeomConstants, "geom_constants", None),
    (ref_gpu.SegmentGPU, "segment_gpu", None),
    (ref_gpu.CircleSegmentGPU, "circle_segment_gpu", None),
    (ref_gpu.LineGPU, "line_gpu", None),
    (ref_gpu.MeshGPU, "mesh_GPU_m", {f: f for f in ("position", "cutting_edge_flag", "fixed_edge_flag", "T_nodes",
                                                    "f", "k", "position_mapping", "node_num_mapping",
                                                    "csr_row_ptr", "csr_col_ind")}),
]
SKIP_FIELDS = {"vptr", "pad", "head", "tail"}


@pytest.mark.skipif(not REF.is_dir() or not Path(NVCC).exists(), reason="needs the reference tree and nvcc")
def test_kernel_parameter_struct_layouts(tmp_path):
    lines = ["#include <cstddef>", "#include <cuda_runtime.h>", "#include <cuda/std/cmath>",
             "#include <thrust/device_vector.h>", '#include "leap_frog.cu"', '#include "grid_gpu_green.h"',
             '#include "tool_gpu.cuh"', '#include "mesh_structure_GPU.h"']
    for cls, cname, members in STRUCTS:
        lines.append(f"static_assert(sizeof({cname}) == {C.sizeof(cls)}, \"size of {cname}\");")
        fields = members or {f: f for f, _ in cls._fields_ if f not in SKIP_FIELDS}
        for py, cpp in fields.items():
            lines.append(f"static_assert(offsetof({cname}, {cpp}) == {getattr(cls, py).offset}, "
                         f"\"offset of {cname}::{cpp}\");")
    src = tmp_path / "layout.cu"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run([NVCC, "-std=c++17", "-w", "-Xcompiler", "-Wno-invalid-offsetof",
                        "-I", str(ROOT / "oracle" / "ref_shim"), "-I", str(REF), "-c", str(src),
                        "-o", str(tmp_path / "layout.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
