"""Edge cases of the fused step on the GPU against the CPU oracle: a single
particle, ragged sizes, an all-blanked state, and a batch of many tiny cases."""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Batch, Solver
from test_gpu_parity import FUSED, compare, pair
from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_side", [1, 2, 37])
def test_tiny_and_ragged_lattices(lib, n_side):
    # 1 and 4 particles (no or few neighbours), 1,369 (no multiple of any block size)
    c = setups.micro(n_side=n_side, seed=5)
    s, o = pair(c)
    for k in range(3):
        s.step()
        o.step()
        compare(s, o, FUSED, what=f"[{n_side}^2 step {k}]")


def test_all_blanked(lib):
    c = setups.micro(n_side=24, seed=6)
    c.particles["blanked"][:] = 1.0
    c.particles["hash"][:] = 0
    s, o = pair(c)
    for k in range(2):
        s.step()
        o.step()
        compare(s, o, FUSED, what=f"[all blanked step {k}]")


def test_fp32k_ragged_matches_fp64(lib):
    c = setups.micro(n_side=37, seed=7)
    a = Solver(c, abi.SPH_PREC_FP64)
    b = Solver(c, abi.SPH_PREC_FP32K)
    a.step(2)
    b.step(2)
    A, B = a.download(["pos", "vel", "S", "rho"]), b.download(["pos", "vel", "S", "rho"])
    for f in A:
        assert rel_err(B[f], A[f]) < 2e-5, f


def tiny_cases(n):
    rng = np.random.default_rng(11)
    out = []
    for k in range(n):
        nx, ny = int(rng.integers(10, 20)), int(rng.integers(6, 10))
        c = setups.cutting(f"tiny{k}", setups.AISI1045, nx, ny, 5e-4, 1.7, float(rng.uniform(100, 400)),
                           float(rng.uniform(0.001, 0.002)), float(rng.uniform(-5, 10)), 5.0, 5e-4, 0.35,
                           s_min=3e-4, s_max=2.5e-3, tool_size=0.008)
        out.append(setups.placed(c, preload_dx=0.3, mode="edge"))
    return out


def test_batch_of_many_tiny_cases(lib):
    cases = tiny_cases(40)
    b = Batch(cases)
    b.step(30)
    assert b.status() & abi.STATUS_BITS["out_of_grid"] == 0
    got = b.download_cases(["pos", "S", "T", "on_seg"])
    red = b.reduce()
    b.close()
    assert np.count_nonzero(red[:, 0]) > 0, "no case made contact"
    for k in (0, 17, 39):
        s = Solver(cases[k], abi.SPH_PREC_FP32K, place_tool=False)
        s.step(30)
        P = s.download(["pos", "S", "T", "on_seg"])
        s.close()
        if k == 0:
            for f in P:
                assert np.array_equal(got[k][f], P[f]), f
        else:
            assert np.array_equal(got[k]["on_seg"], P["on_seg"])
            for f in ("pos", "S", "T"):
                assert rel_err(got[k][f] - (300.0 if f == "T" else 0.0), P[f] - (300.0 if f == "T" else 0.0)) < 1e-5, (k, f)
