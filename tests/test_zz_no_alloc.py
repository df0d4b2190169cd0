"""The allocation-free CG + Jacobi entry point, called through the C ABI, against gdt_solve.

gdt_solve_cg_jacobi_noalloc serves callers that may not allocate device memory (a host framework
that owns all device memory through its own pool, or a loop that cannot take cudaMalloc's implicit
synchronisation): its work vectors sit in a fixed device array of the library, which keeps the last
call's contents between calls. Two calls in a row must both agree with the allocating solver and
with a direct sparse solve on the host, and the second call must leave the device's free memory
unchanged (the first call on a device may load the library's module, which places the array).
This file is collected last on purpose, so a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _system(gdt, cells=160):
    g = gdt.make_cube_grid([0, 0], [1, 1], [cells, cells], simplex=True)
    rng = np.random.default_rng(42)
    kappa = torch.tensor(np.exp(rng.standard_normal(g.num_elements)), device="cuda")
    prob = gdt.DiffusionProblem(g)
    prob.assemble(kappa)
    return prob


def test_noalloc_solve_matches_gdt_solve_twice(gdt):
    prob = _system(gdt)
    op = prob.op
    n = prob.space.num_DoFs
    assert n <= 262144
    tol = 1e-12
    ref = op.apply_inverse(prob.rhs, opts={"type": "cg", "precond": "jacobi", "tol": tol})
    rp, col, val = op.csr()
    L = gdt._capi.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    A = sp.csr_matrix((val.cpu().numpy(), col.cpu().numpy(), rp.cpu().numpy()), shape=(n, n))
    direct = spl.spsolve(A.tocsc(), prob.rhs.cpu().numpy())
    free = []
    for call in range(2):
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        info = gdt._capi.SolveInfo()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = L.gdt_solve_cg_jacobi_noalloc(C.c_void_p(rp.data_ptr()), C.c_void_p(col.data_ptr()),
                                           C.c_void_p(val.data_ptr()), C.c_int64(n),
                                           C.c_void_p(prob.rhs.data_ptr()), C.c_void_p(x.data_ptr()),
                                           C.c_double(tol), 100000, stream, C.byref(info))
        torch.cuda.synchronize()
        free.append((free_before, torch.cuda.mem_get_info()[0]))
        assert st == gdt._capi.OK, f"call {call}: status {st}"
        assert info.converged == 1
        assert abs(info.iterations - op.last_solve_info["iterations"]) <= 2
        err = ((x - ref).abs().max() / ref.abs().max()).item()
        assert err < 1e-10, f"call {call}: relative difference {err} to gdt_solve"
        xd = x.cpu().numpy()
        err_direct = np.abs(xd - direct).max() / np.abs(direct).max()
        assert err_direct < 1e-10, f"call {call}: relative difference {err_direct} to the direct solve"
    # the second call allocates nothing: the device's free memory is the same before and after it
    assert free[1][0] == free[1][1], f"free device memory changed during the second call: {free[1]}"


def test_noalloc_rejects_systems_above_its_maximum(gdt):
    prob = _system(gdt, cells=16)
    rp, col, val = prob.op.csr()
    L = gdt._capi.load()
    x = torch.zeros(prob.space.num_DoFs, dtype=torch.float64, device="cuda")
    # the size check comes before any device work, so the small arrays are never read past their end
    st = L.gdt_solve_cg_jacobi_noalloc(C.c_void_p(rp.data_ptr()), C.c_void_p(col.data_ptr()),
                                       C.c_void_p(val.data_ptr()), C.c_int64(262145),
                                       C.c_void_p(prob.rhs.data_ptr()), C.c_void_p(x.data_ptr()),
                                       C.c_double(1e-10), 100, None, None)
    assert st == gdt._capi.EINVAL
