"""Host side of the batched context: the case generator, tool placement on
the host and argument checks of sph_batch_create (no GPU needed)."""
import ctypes as C
import math

import numpy as np

from sph_fem_2d_cutting_gpu_gb300 import abi, setups


def test_placed_tool_matches_reference_placement(lib):
    # benchmarks_NZ.cpp:247-267: right point 0.01 dx left of the workpiece,
    # lowest point at the target uncut chip thickness below its top
    c = setups.small_cut()
    p = setups.placed(c)
    st = abi.tool_model_host(p)["state"]
    dx = c.info["dx"]
    assert math.isclose(st.right_point, c.info["lo_x"] - 0.01 * dx, rel_tol=0, abs_tol=1e-12)
    assert math.isclose(c.info["hi_y"] - st.lowest_point, c.feed, rel_tol=0, abs_tol=1e-12)
    assert p.tool_mesh["nodes"].flags["C_CONTIGUOUS"]
    assert c.tool_mesh["nodes"] is not p.tool_mesh["nodes"]


def test_batched_sweep_draws(lib):
    cases = setups.batched_sweep(n_cases=6, seed=3)
    assert len(cases) == 6
    for c in cases:
        assert c.info["ny"] == 200
        assert 20_000 * 0.99 <= c.N <= 300_000 * 1.01
        assert 30.0 <= c.info["speed_mpmin"] <= 300.0
        assert 20e-4 <= c.feed <= 150e-4
        assert -10.0 <= c.info["rake"] <= 15.0
        assert 1500 <= c.info["nodes"] <= 10_000
        assert c.dt > 0
    again = setups.batched_sweep(n_cases=6, seed=3)
    assert [c.N for c in again] == [c.N for c in cases]


def test_batch_create_argument_checks(lib):
    cases = [setups.placed(setups.small_cut())]
    descs = (abi.CaseDesc * 1)()
    host = abi.particles_struct(cases[0].particles, cases[0].N)
    tool, keep = cases[0].tool_struct()
    d = descs[0]
    d.host = C.pointer(host)
    d.tool = C.pointer(tool)
    d.dt = cases[0].dt
    d.bbmin[0], d.bbmin[1] = cases[0].grid.bbmin[0], cases[0].grid.bbmin[1]
    d.bbmax[0], d.bbmax[1] = cases[0].grid.bbmax[0], cases[0].grid.bbmax[1]
    ctx = C.c_void_p()
    c0 = cases[0].constants
    g = cases[0].grid
    # an unknown precision form; zero cases; bad time step
    assert lib.sph_batch_create(C.byref(c0), C.byref(g), 1, descs, 7, 0, C.byref(ctx)) == abi.SPH_ERR_INVALID
    assert lib.sph_batch_create(C.byref(c0), C.byref(g), 0, descs, abi.SPH_PREC_FP32K, 0, C.byref(ctx)) == \
        abi.SPH_ERR_INVALID
    d.dt = 0.0
    assert lib.sph_batch_create(C.byref(c0), C.byref(g), 1, descs, abi.SPH_PREC_FP32K, 0, C.byref(ctx)) == \
        abi.SPH_ERR_INVALID
    assert not ctx.value
    del keep
