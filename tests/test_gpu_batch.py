"""Batched multi-case context on the GPU, against single-case contexts.

Case 0 of a batch sits at offset (0, 0) of the global grid and sees the same
cell geometry as a single-case context on its own box, so its results are
bit-identical.  Cases k > 0 are moved by their offsets: their positions,
tool nodes and cell-corner coordinates differ from a single-case run by the
rounding of that translation, so they are compared within a tolerance.
"""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Batch, Solver
from conftest import rel_err

pytestmark = pytest.mark.gpu

STATE = ["pos", "vel", "rho", "S", "T", "eps_pl", "eps_pl_dot", "fc", "ft", "n"]
EXACT = ["on_seg", "blanked", "fixed", "tool_particle"]
STEPS = 60
# cases k > 0: translation rounding (~1e-16 of the offset) through FP32 cell
# coordinates grows over the steps; norm-wise bound on every state field
RTOL_SHIFTED = 1e-5


def small_cases():
    spec = [  # nx, ny, speed m/min, uncut chip thickness cm, rake deg
        (40, 16, 300.0, 0.002, 0.0),
        (56, 20, 180.0, 0.003, 8.0),
        (32, 12, 420.0, 0.0015, -6.0),
    ]
    cases = []
    for k, (nx, ny, v, feed, rake) in enumerate(spec):
        c = setups.cutting(f"batch{k}", setups.AISI1045, nx, ny, 5e-4, 1.7, v, feed, rake, 5.0, 5e-4, 0.35,
                           s_min=2e-4, s_max=2.5e-3, tool_size=0.015)
        cases.append(setups.placed(c, preload_dx=0.3))
    return cases


PRECISIONS = pytest.mark.parametrize("prec", [abi.SPH_PREC_FP32K, abi.SPH_PREC_FP64], ids=["fp32k", "fp64"])


def single_run(case, steps, prec=abi.SPH_PREC_FP32K):
    s = Solver(case, prec, place_tool=False)
    s.step(steps)
    P = s.download(STATE + EXACT)
    red = np.concatenate([s.reduce_force(), [s.max_T()]])
    T = s.fem()["T"]
    s.close()
    return P, red, T


@PRECISIONS
def test_batch_of_one_is_bit_identical(lib, prec):
    case = small_cases()[0]
    b = Batch([case], prec)
    b.step(STEPS)
    got = b.download_cases(STATE + EXACT)[0]
    red = b.reduce()[0]
    T = b.fem_T()[0]
    b.close()
    P, red1, T1 = single_run(case, STEPS, prec)
    for f in STATE + EXACT:
        assert np.array_equal(got[f], P[f]), f"{f}: {np.count_nonzero(got[f] != P[f])} entries differ"
    assert np.array_equal(T, T1)
    assert np.array_equal(red, red1)


@PRECISIONS
def test_batch_cases_match_single_runs(lib, prec):
    """Every case runs with its own time step and tool velocity (in both forms)."""
    cases = small_cases()
    b = Batch(cases, prec)
    assert b.info[0]["offset"].tolist() == [0.0, 0.0]
    b.step(STEPS)
    assert b.status() & abi.STATUS_BITS["out_of_grid"] == 0
    got = b.download_cases(STATE + EXACT)
    red = b.reduce()
    Ts = b.fem_T()
    b.close()
    for k, case in enumerate(cases):
        P, red1, T1 = single_run(case, STEPS, prec)
        assert got[k]["pos"].shape == P["pos"].shape
        if k == 0:
            for f in STATE + EXACT:
                assert np.array_equal(got[k][f], P[f]), f"case 0 {f}"
            assert np.array_equal(Ts[k], T1)
            assert np.array_equal(red[k], red1)
            continue
        for f in EXACT:
            assert np.array_equal(got[k][f], P[f]), f"case {k} {f}"
        for f in STATE:
            e = rel_err(got[k][f], P[f])
            assert e <= RTOL_SHIFTED, f"case {k} {f}: {e:.3e}"
        assert rel_err(Ts[k] - 300.0, T1 - 300.0) <= RTOL_SHIFTED
        assert rel_err(red[k][:2], red1[:2]) <= RTOL_SHIFTED
        assert abs(red[k][2] - red1[2]) <= RTOL_SHIFTED * max(red1[2] - 300.0, 1.0)


def test_batch_reduce_matches_download(lib):
    cases = small_cases()
    b = Batch(cases)
    for steps in (0, 7):
        if steps:
            b.step(steps)
        red = b.reduce()
        per = b.download_cases(["fc", "ft", "T", "blanked"])
        for k, d in enumerate(per):
            f = (d["fc"] + d["ft"]).sum(0)
            assert np.allclose(red[k][:2], f, rtol=1e-12, atol=1e-300)
            live = d["blanked"] != 1.0
            assert red[k][2] == d["T"][live].max()
    b.close()


def test_batch_rejects_single_case_calls(lib):
    b = Batch(small_cases()[:2])
    for name in ("sph_predict", "sph_correct", "sph_plasticity_johnson_cook", "sph_step_staged",
                 "sph_compute_contact_forces_fem", "sph_material_fric_heat_gen_fem"):
        assert getattr(b.lib, name)(b.ctx) == abi.SPH_ERR_STATE, name
    assert b.lib.sph_set_dt(b.ctx, 1e-4) == abi.SPH_ERR_STATE
    assert b.lib.sph_set_tool_velocity(b.ctx, 1.0, 0.0) == abi.SPH_ERR_STATE
    b.close()
