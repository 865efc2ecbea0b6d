"""The AISI 1045 cut of config 3 against the CPU oracle and FP32K against FP64.

1. The full-size cut (1600 x 400 = 640,000 particles, tool of about 20,000
   nodes, edge placement) in the plain FP64 form: after 3,000 fused steps
   (contact established, the chip root heated), a window of 200 consecutive
   steps in which every GPU step is compared with one oracle step from the
   same start-of-step state (particles, segments, FEM temperatures, tool
   kinematics): index work bit for bit, FP64 fields within 1e-10 norm-wise.
2. A reduced cut of the same material and tool geometry (400 x 100
   particles): FP32K against FP64 over 3,000 steps, cutting force within 1 %
   of the peak force and peak temperature within 1 % of its rise, at every
   checkpoint (the bench runs the full-size comparison over 20,000 steps).
"""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver
from oracle.oracle import OracleSim
from conftest import rel_err

pytestmark = pytest.mark.gpu

RTOL = 1e-10
FIELDS = ["pos", "vel", "rho", "S", "T", "eps_pl", "eps_pl_dot", "p", "R", "fc", "ft", "n", "h"]
RATES = ["pos_t", "vel_t", "rho_t", "S_t", "T_t"]
EXACT = ["hash", "idx", "on_seg", "blanked", "fixed", "tool_particle"]
WARM = 3000
WINDOW = 200


def test_config3_fp64_window_matches_oracle_per_step(lib):
    case = setups.placed(setups.aisi1045_cut(), mode="edge")
    assert case.N == 640_000 and case.info["nodes"] > 19_000
    s = Solver(case, abi.SPH_PREC_FP64, place_tool=False)
    s.step(WARM)
    P = s.download()
    assert np.abs(P["fc"]).max() > 0, "no contact after the warm-up"
    worst = {}
    for k in range(WINDOW):
        ts = s.tool_state()
        o = OracleSim(case.constants, case.grid, P, case.dt,
                      tool=dict(segments=s.segments(), fem=s.fem(), state=ts, n_cut_colors=ts.n_cut_colors))
        o.step()
        s.step()
        P = s.download()
        act = o.P["blanked"] != 1.0
        for f in EXACT:
            assert np.array_equal(P[f], o.P[f]), f"step {WARM + k + 1} {f}: {np.count_nonzero(P[f] != o.P[f])} differ"
        for f in FIELDS + RATES:
            a, b = (P[f][act], o.P[f][act]) if f in RATES else (P[f], o.P[f])
            e = rel_err(a, b)
            worst[f] = max(worst.get(f, 0.0), e)
            assert e <= RTOL, f"step {WARM + k + 1} {f}: relative error {e:.3e}"
        seg, fem = s.segments(), s.fem()
        assert np.array_equal(seg["left"], o.seg["left"]) and np.array_equal(seg["right"], o.seg["right"])
        assert rel_err(seg["heat_exchange"], o.seg["heat_exchange"]) <= RTOL
        assert rel_err(fem["T"], o.fem["T"]) <= RTOL
    assert s.status() == 0
    print(f"\n[config 3 FP64 window, steps {WARM + 1}-{WARM + WINDOW}] worst relative error per field: "
          + ", ".join(f"{f} {e:.1e}" for f, e in worst.items()))


def reduced_cut():
    c = setups.cutting("aisi1045_reduced", setups.AISI1045, 400, 100, 2.5e-4, 1.7, 120.0, 0.01, -6.0, 5.0, 2e-3,
                       0.35, s_min=1e-4, s_max=2.5e-3, tool_size=0.05)
    return setups.placed(c, mode="edge")


def curve(case, precision, steps, every):
    s = Solver(case, precision, place_tool=False)
    h = []
    for _ in range(steps // every):
        s.step(every)
        h.append((*s.reduce_force(), s.max_T()))
    st = s.status()
    s.close()
    return np.array(h), st


def test_reduced_cut_fp32k_within_one_percent_of_fp64(lib):
    case = reduced_cut()
    h64, st64 = curve(case, abi.SPH_PREC_FP64, 3000, 250)
    h32, st32 = curve(case, abi.SPH_PREC_FP32K, 3000, 250)
    assert st64 == 0 and st32 == 0
    fmax = np.hypot(h64[:, 0], h64[:, 1]).max()
    assert fmax > 0, "no cutting force developed"
    rise = max(h64[:, 2].max() - 300.0, 1.0)
    ef = np.hypot(h32[:, 0] - h64[:, 0], h32[:, 1] - h64[:, 1]).max() / fmax
    eT = np.abs(h32[:, 2] - h64[:, 2]).max() / rise
    assert ef <= 0.01, f"cutting force deviates {ef:.3e} of the peak force"
    assert eT <= 0.01, f"peak temperature deviates {eT:.3e} of the temperature rise"
