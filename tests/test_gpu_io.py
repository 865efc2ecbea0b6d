"""Pipelined host I/O: the asynchronous upload/download calls give the same
results as the synchronous ones, and the ordering rules hold."""
import ctypes as C

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver

pytestmark = pytest.mark.gpu

STATE = ["pos", "vel", "h", "rho", "S", "fc", "ft", "n", "fixed", "blanked", "tool_particle", "eps_pl",
         "eps_pl_dot", "T", "pos_t", "vel_t", "rho_t", "S_t", "T_t", "on_seg", "hash"]


def pinned_like(arrays):
    import torch
    out, keep = {}, []
    for k, v in arrays.items():
        t = torch.empty(v.shape, dtype=torch.float64 if v.dtype == np.float64 else torch.int32, pin_memory=True)
        a = t.numpy()
        a[...] = v
        out[k] = a
        keep.append(t)
    return out, keep


@pytest.mark.parametrize("precision", [abi.SPH_PREC_FP64, abi.SPH_PREC_FP32K])
def test_pipelined_steps_equal_synchronous(lib, precision):
    # no tool: a step's result depends on the particle state alone (a tool's position
    # and FEM temperatures live in the context and advance with every step)
    case = setups.micro(n_side=48, seed=12)
    s = Solver(case, precision)
    s.step(5)
    state = s.download(STATE)
    # synchronous reference: the state in, one step, the result out
    s.upload(state)
    s.step()
    want = s.download(STATE)
    # pipelined: six requests on the same input state (the three particle buffers
    # rotate twice)
    src, keep_in = pinned_like(state)
    outs = [pinned_like(state) for _ in range(6)]
    pin_in = abi.particles_struct(src, case.N)
    pin_out = [abi.particles_struct(o, case.N) for o, _ in outs]
    s.upload_async(pin_in)
    for k in range(6):
        s.step()
        s.download_async(pin_out[k])
        if k < 5:
            s.upload_async(pin_in)
    s.sync()
    # and a synchronous step afterwards still sees consistent state
    s.upload(state)
    s.step()
    again = s.download(STATE)
    for f in STATE:
        assert np.array_equal(again[f], want[f]), f
    for o, _ in outs:
        for f in STATE:
            assert np.array_equal(o[f], want[f]), f
    s.close()


def test_async_upload_refuses_derived_fields(lib):
    case = setups.micro(n_side=16)
    s = Solver(case, abi.SPH_PREC_FP32K)
    P = s.download(["pos", "p"])
    st = abi.particles_struct(P, case.N)
    assert s.lib.sph_upload_particles_async(s.ctx, C.byref(st)) == abi.SPH_ERR_INVALID
    s.close()
