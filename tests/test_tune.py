"""Launch shapes and the autotuner."""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups, tune
from sph_fem_2d_cutting_gpu_gb300.solver import Solver
from conftest import rel_err


def test_launch_variants_listed(lib):
    v = tune.launch_variants()
    assert v[0] == (128, 6, 0, 1)     # the default: 24 resident warps per SM, no spills
    assert len(v) >= 4 and len(set(v)) == len(v)
    assert any(c > 0 for _, _, c, _ in v) and any(l > 1 for _, _, _, l in v)
    for block, min_blocks, staged, lanes in v:
        assert block % 32 == 0 and block * min_blocks <= 2048
        assert 32 % lanes == 0 and (lanes == 1 or staged == 0)
        # staged records + pair lists fit the 227 KB a block may use
        assert staged * 64 + 32 * block * 4 <= 227 * 1024


def test_with_geometry_copies_grid():
    c = setups.small_cut()
    c2 = tune.with_geometry(c, 2, 1)
    assert (c2.grid.cell_factor, c2.grid.stencil) == (2, 1)
    assert (c.grid.cell_factor, c.grid.stencil) == (1, 2)
    assert c2.grid.bbmin[0] == c.grid.bbmin[0]


def run_variants(case, steps, fields):
    out = []
    for v in range(len(tune.launch_variants())):
        s = Solver(case, abi.SPH_PREC_FP32K, place_tool=False)
        tune.set_variant(s, v)
        s.step(steps)
        out.append(s.download(fields))
        s.close()
    return out


@pytest.mark.gpu
def test_launch_variants_agree_without_tool(lib):
    # each particle's sums run in one thread in the same neighbour order
    # whatever the launch shape (or, with several lanes per particle, in
    # interleaved partial sums merged by a compensated two-sum), and the cell
    # lists are identical; the register budget of a shape changes the compiled
    # FP32 code (which multiply-adds are fused), so results agree to FP32
    # rounding
    runs = run_variants(setups.micro(n_side=128, seed=3), 3, ["pos", "vel", "S", "rho", "T", "eps_pl", "hash"])
    for v, P in enumerate(runs[1:], 1):
        assert np.array_equal(P["hash"], runs[0]["hash"]), v
        for f in ("pos", "vel", "S", "rho", "T", "eps_pl"):
            assert rel_err(P[f], runs[0][f]) < 1e-5, (v, f)


@pytest.mark.gpu
def test_launch_variants_agree_with_tool(lib):
    # with a tool the friction heat of a segment is an FP64 atomic sum whose
    # order follows the launch shape: agreement to rounding
    case = setups.placed(setups.small_cut(nx=48, ny=20), preload_dx=0.3)
    runs = run_variants(case, 40, ["pos", "vel", "S", "T", "eps_pl", "fc", "ft"])
    for v, P in enumerate(runs[1:], 1):
        for f in P:
            assert rel_err(P[f], runs[0][f]) < 1e-6, (v, f)


@pytest.mark.gpu
def test_autotune_returns_fastest(lib):
    case = setups.micro(n_side=256)
    best, table = tune.autotune(lambda c: Solver(c, abi.SPH_PREC_FP32K), case, warmup=3, steps=5)
    assert len(table) == len(tune.CELL_GEOMETRIES) * (len(tune.launch_variants()) + 1)
    assert sum(r["step_form"] == abi.SPH_STEP_PERSISTENT for r in table) == len(tune.CELL_GEOMETRIES)
    assert best["ms_per_step"] == min(r["ms_per_step"] for r in table)


@pytest.mark.gpu
def test_split_lanes_keep_the_non_finite_stencil_rule(lib):
    """A NaN in a record spreads through its stencil with the reference's zero
    weights; with several lanes per particle the stencil's marks are combined
    before the rerun, so the same particles are blanked as with one lane."""
    c = setups.micro(n_side=48, seed=6)
    c.particles["vel"][100, 0] = np.nan
    c.particles["S"][500, 1] = np.inf
    lanes = [v for v, sh in enumerate(tune.launch_variants()) if sh[3] > 1]
    assert lanes
    out = []
    for v in [0] + lanes:
        s = Solver(c, abi.SPH_PREC_FP32K)
        tune.set_variant(s, v)
        s.step(2)
        out.append((s.download(["blanked", "pos", "rho"]), s.status()))
        s.close()
    P0, st0 = out[0]
    assert st0 & abi.STATUS_BITS["nan_blanked"] and (P0["blanked"] == 1.0).sum() >= 3
    for (P, st), v in zip(out[1:], lanes):
        assert np.array_equal(P["blanked"], P0["blanked"]), v
        live = P0["blanked"] != 1.0
        assert rel_err(P["pos"][live], P0["pos"][live]) < 1e-6, v
