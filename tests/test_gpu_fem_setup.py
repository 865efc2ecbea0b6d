"""The FEM tool's thermal system assembled on the device (a context's set-up):
element stiffness and lumped mass colour by colour, the Dirichlet elimination
and the lumped inverse (FEM_thermal_gpu.cu:126-332).

- bit for bit the host assembly of the tool model (the host export the CPU
  oracle uses): the same element routine, the same summation order;
- within 1e-13 of the reference's own kernels (do_stiffness_mass_matrix_
  construction_p1q3, do_dirichlet_bdc_p1q3, do_inverse_mass_matrix_lumped, from
  the cubin of the unmodified FEM_thermal_gpu.cu) run on the same mesh, colouring
  and CSR pattern: their element matrices go through GLM products and
  inverses, a different operation order.  The reference's Dirichlet threads of
  one colour race on shared symmetric entries; the right-hand side at fixed
  nodes ends at T0 in every order, and the rest is compared.
"""
import ctypes as C

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver
from conftest import rel_err

pytestmark = pytest.mark.gpu

CASES = ["small_cut", "ti64_cut"]


@pytest.mark.parametrize("name", CASES)
def test_device_assembly_is_the_host_assembly(lib, name):
    case = getattr(setups, name)()
    host = abi.tool_model_host(case)["fem"]
    s = Solver(case, place_tool=False)
    dev = s.fem()
    s.close()
    for k in ("row_ptr", "col_ind", "K", "M_inv", "f"):
        assert np.array_equal(dev[k], host[k]), f"{k}: {np.count_nonzero(dev[k] != host[k])} entries differ"


@pytest.mark.parametrize("name", CASES)
def test_device_assembly_matches_the_reference_kernels(lib, name):
    torch = pytest.importorskip("torch")
    from oracle import ref_gpu
    try:
        fem_mod = ref_gpu.RefModule("fem")
    except FileNotFoundError:
        pytest.skip("reference cubins not built")
    case = getattr(setups, name)()
    tm = abi.tool_model_host(case)
    host = tm["fem"]
    s = Solver(case, place_tool=False)
    dev = s.fem()
    s.close()
    el = np.ascontiguousarray(tm["elements"])
    ne, nn, nz = len(el), len(host["T"]), len(host["K"])
    ffl = np.ascontiguousarray(case.tool_mesh["fixed_flags"], np.int32)          # int3 per element
    fixed = np.flatnonzero(ffl.any(1)).astype(np.int32)
    cuda = torch.device("cuda", 0)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    pos, elements, row_ptr, col_ind = d(host["position"]), d(el), d(host["row_ptr"]), d(host["col_ind"])
    flags, fixed_d = d(ffl), d(fixed)
    M = torch.zeros(nn, dtype=torch.float64, device=cuda)
    K = torch.zeros(nz, dtype=torch.float64, device=cuda)
    f = torch.zeros(nn, dtype=torch.float64, device=cuda)
    T = torch.zeros(nn, dtype=torch.float64, device=cuda)
    M_inv = torch.zeros(nn, dtype=torch.float64, device=cuda)
    P = ref_gpu.ptr
    fem_mod.launch("ref_set_fem_constants", 1, case.constants.tool, block=1)
    ncol = tm["n_colors"]
    for c in range(1, ncol + 1):   # FEM_thermal_2D_GPU::stiffness_mass_matrix_construction
        fem_mod.launch("do_stiffness_mass_matrix_construction_p1q3", ne, C.c_int32(c), C.c_int32(ne), P(pos),
                       P(elements), P(row_ptr), P(col_ind), C.c_int32(ncol), P(M), P(K))
    for c in range(1, ncol + 1):   # dirichlet_bdc
        fem_mod.launch("do_dirichlet_bdc_p1q3", len(fixed), C.c_int32(c), C.c_int32(len(fixed)), C.c_int32(ncol),
                       P(pos), P(elements), P(flags), P(fixed_d), P(row_ptr), P(col_ind), P(M), P(K), P(f), P(T))
    fem_mod.launch("do_inverse_mass_matrix_lumped", nn, C.c_int32(nn), P(M_inv), P(M))
    torch.cuda.synchronize()
    Kr, Mr, fr = K.cpu().numpy(), M_inv.cpu().numpy(), f.cpu().numpy()
    assert rel_err(dev["K"], Kr) <= 1e-13
    assert rel_err(dev["M_inv"], Mr) <= 1e-13
    fixed_nodes = np.zeros(nn, bool)
    for e in fixed:
        a, b, cc = el[e, :3]
        fx, fy, fz = ffl[e]
        fixed_nodes[[a, b]] |= bool(fx)
        fixed_nodes[[b, cc]] |= bool(fy)
        fixed_nodes[[cc, a]] |= bool(fz)
    assert fixed_nodes.any()
    assert np.all(dev["f"][fixed_nodes] == case.constants.tool.T0)
    free = ~fixed_nodes
    assert rel_err(dev["f"][free], fr[free], scale=np.abs(fr).max()) <= 1e-13
