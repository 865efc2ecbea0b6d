"""Run-level parity: the Ti6Al4V orthogonal cut (200 x 60 particles, dx = 5 um,
tool mesh of about 2,000 nodes, 70 m/min, 2,000 steps) on the GPU against the
CPU oracle.  Cutting force sum(fc + ft) and peak temperature are compared at
checkpoints over the whole run: within 2 % for the plain FP64 form, within
1 % for the FP32-compensated form (force relative to the run's peak force,
temperature on the rise above 300 K)."""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu

STEPS = 2000
EVERY = 100


def force_T(P):
    f = (P["fc"] + P["ft"]).sum(0)
    act = P["blanked"] != 1.0
    return f, float(P["T"][act].max())


@pytest.fixture(scope="module")
def oracle_run(lib):
    c = setups.ti64_cut(steps=STEPS)
    s = Solver(c)                      # builds and places the tool
    ts = s.tool_state()
    o = OracleSim(c.constants, c.grid, s.download(), c.dt,
                  tool=dict(segments=s.segments(), fem=s.fem(), state=ts, n_cut_colors=ts.n_cut_colors))
    s.close()
    hist = []
    for k in range(1, STEPS + 1):
        o.step()
        if k % EVERY == 0:
            hist.append(force_T(o.P))
    return c, hist


def gpu_run(c, precision):
    s = Solver(c, precision)
    hist = []
    for k in range(STEPS // EVERY):
        s.step(EVERY)
        P = s.download(["fc", "ft", "T", "blanked"])
        hist.append(force_T(P))
    st = s.status()
    s.close()
    return hist, st


def compare(hist_g, hist_o, tol):
    fo = np.array([h[0] for h in hist_o])
    fg = np.array([h[0] for h in hist_g])
    To = np.array([h[1] for h in hist_o])
    Tg = np.array([h[1] for h in hist_g])
    fmax = np.abs(fo).max()
    assert fmax > 0, "no contact force developed"
    ef = np.abs(fg - fo).max() / fmax
    rise = max(To.max() - 300.0, 1.0)
    eT = np.abs(Tg - To).max() / rise
    return ef, eT


@pytest.mark.parametrize("precision,tol", [(abi.SPH_PREC_FP64, 0.02), (abi.SPH_PREC_FP32K, 0.01)])
def test_ti64_run_force_and_peak_temperature(oracle_run, precision, tol):
    c, hist_o = oracle_run
    hist_g, st = gpu_run(c, precision)
    ef, eT = compare(hist_g, hist_o, tol)
    assert ef <= tol, f"cutting force deviates {ef:.3e} of the peak force"
    assert eT <= tol, f"peak temperature deviates {eT:.3e} of the temperature rise"
