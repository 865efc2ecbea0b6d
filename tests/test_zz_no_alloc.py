"""GPU test of sph_cells_build_noalloc, the cell-list build that allocates
nothing (for callers that cannot call cudaMalloc when they need a cell
list).  Its output must equal the allocating path (sph_assign_hashes +
sph_sort on a context) on two calls in a row, which share the fixed scratch.
This file is collected last so a failure here comes after every other test.
"""
import ctypes as C

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _compare_with_context_sort(lib, c):
    """Run the allocating path (sph_assign_hashes + sph_sort on a context) and
    sph_cells_build_noalloc twice on the same particles; both calls must give
    its permutation, sorted hashes and cell tables bit for bit."""
    torch = pytest.importorskip("torch")
    s = Solver(c)
    g = s.geometry()
    assert c.N <= 262144 and g.num_cell <= 262143
    host = s.download(["pos", "blanked", "hash"])
    s.assign_hashes()
    s.sort()
    s.status()      # out-of-grid particles raise a status bit on the allocating path
    ref = s.download(["idx", "hash"])
    ref_start, ref_end = s.cells()
    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(host["pos"]).to(dev)
    blanked = torch.from_numpy(host["blanked"]).to(dev)
    err = C.create_string_buffer(256)
    for call in range(2):
        hash_io = torch.from_numpy(host["hash"]).to(dev)
        perm = torch.full((c.N,), -5, dtype=torch.int32, device=dev)
        hsorted = torch.full((c.N,), -5, dtype=torch.int32, device=dev)
        cstart = torch.full((g.num_cell,), -7, dtype=torch.int32, device=dev)
        cend = torch.full((g.num_cell,), -7, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        r = lib.sph_cells_build_noalloc(C.c_void_p(pos.data_ptr()), C.c_void_p(blanked.data_ptr()),
                                        C.c_void_p(hash_io.data_ptr()), c.N, C.byref(g),
                                        C.c_void_p(perm.data_ptr()), C.c_void_p(hsorted.data_ptr()),
                                        C.c_void_p(cstart.data_ptr()), C.c_void_p(cend.data_ptr()), None, err, 256)
        torch.cuda.synchronize()
        assert r == abi.SPH_OK, err.value.decode()
        assert np.array_equal(perm.cpu().numpy(), ref["idx"]), f"call {call}: permutation differs"
        assert np.array_equal(hsorted.cpu().numpy(), ref["hash"]), f"call {call}: sorted hash differs"
        cs = cstart.cpu().numpy()
        assert np.array_equal(cs, ref_start), f"call {call}: cell_start differs"
        ne = cs != -1
        assert np.array_equal(cend.cpu().numpy()[ne], ref_end[ne]), f"call {call}: cell_end differs"
        assert np.all(cend.cpu().numpy()[~ne] == -7), "cell_end of empty cells must stay untouched"
    s.close()
    return g


def _shuffled_micro(n_side, seed):
    c = setups.micro(n_side=n_side, seed=seed)
    rng = np.random.default_rng(seed + 100)
    perm_in = rng.permutation(c.N)
    c.particles = {k: np.ascontiguousarray(v[perm_in]) for k, v in c.particles.items()}
    return c, rng


def test_noalloc_cell_build_matches_context_sort(lib):
    c, _ = _shuffled_micro(160, 21)
    c.particles["blanked"][::11] = 1.0
    c.particles["hash"][::11] = 7          # stale hash of blanked particles (a valid cell)
    _compare_with_context_sort(lib, c)


def test_noalloc_out_of_grid_and_stale_hashes(lib):
    """Particles outside the grid and blanked particles whose stale hash lies
    outside the cell range all go to the trailing bucket, in original-index
    order, on both paths."""
    c, rng = _shuffled_micro(160, 22)
    P = c.particles
    g = c.grid
    out = rng.choice(c.N, 300, replace=False)
    P["pos"][out[:100], 0] = g.bbmin[0] - rng.uniform(1e-3, 1e-2, 100)     # left of the grid
    P["pos"][out[100:200], 1] = g.bbmin[1] - rng.uniform(1e-3, 1e-2, 100)  # below it
    P["blanked"][out[200:250]] = 1.0
    P["hash"][out[200:250]] = -1                                            # stale, below the range
    P["blanked"][out[250:]] = 1.0
    P["hash"][out[250:]] = 10 ** 7                                          # stale, above the range
    _compare_with_context_sort(lib, c)


def test_noalloc_at_the_size_limits(lib):
    """262,144 particles (the maximum) on a grid of just under 262,143 cells,
    so the single-block scan covers its last buckets."""
    c, rng = _shuffled_micro(512, 23)
    g = c.grid
    edge = g.h * g.cell_factor
    nx = int(np.ceil((g.bbmax[0] - g.bbmin[0] + 2e-6) / edge))
    ny = 262143 // nx
    g.bbmax[1] = g.bbmin[1] + (ny - 0.5) * edge - 2e-6     # ceil gives ny rows
    c.particles["blanked"][::97] = 1.0
    c.particles["hash"][::97] = nx * ny + 5                 # stale, outside the range
    geo = _compare_with_context_sort(lib, c)
    assert geo.num_cell > 262143 - nx, geo.num_cell


def test_noalloc_rejects_sizes_beyond_the_scratch(lib):
    g = abi.GeomConstants()
    g.nx, g.ny, g.num_cell, g.dx, g.stencil = 10, 10, 100, 1.0, 2
    err = C.create_string_buffer(256)
    dummy = C.c_void_p(16)      # never dereferenced: sizes are checked before any device work
    r = lib.sph_cells_build_noalloc(dummy, dummy, dummy, 262145, C.byref(g), dummy, None, dummy, dummy, None, err, 256)
    assert r == abi.SPH_ERR_INVALID
    assert b"262144" in err.value
    g.num_cell = 262144
    r = lib.sph_cells_build_noalloc(dummy, dummy, dummy, 1000, C.byref(g), dummy, None, dummy, dummy, None, err, 256)
    assert r == abi.SPH_ERR_INVALID
