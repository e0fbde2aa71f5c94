"""yk_cg_solve_static (the allocation-free FP64 solve) against yk_cg_solve.

Collected last on purpose: it must pass both alone and after every other
test of the session.  Two consecutive calls of the static entry point on the
same inputs must each agree with the context solve to 1e-12 relative (same
algorithm, same arithmetic: the results are expected to be identical).  The
free device memory (cudaMemGetInfo) must not move across the second call,
and across the first only by the library's fixed scratch array.  A lattice
beyond the static scratch is refused with YK_EINVAL.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the static scratch array (6.6 MB) rounded up to the 2 MiB granularity of
# device memory, plus one more granule for the module that holds it
STATIC_BYTES_BOUND = 10 << 20


def _params(yk, Nt, Nx):
    return yk.Params.default(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=0.5, fermion_mass=0.1, wilson_param=1.0,
                             Nt=Nt, Nx=Nx, cg_tol=1e-12, cg_tol_mode=yk.YK_TOL_REL, seed=1234,
                             init=yk.YK_INIT_PHILOX)


@pytest.mark.parametrize("Nt,Nx,mtype", [(32, 32, 0), (128, 128, 1), (6, 10, 1)])
def test_static_solve_matches_context_solve(ylib, cuda, Nt, Nx, mtype):
    yk, torch = ylib, cuda
    p = _params(yk, Nt, Nx)
    a = p.action()
    rng = np.random.default_rng(11)
    V = Nt * Nx
    with yk.Context(p) as ctx:
        ctx.set_field(rng.uniform(-1, 1, V))
        b = rng.normal(size=(V, 4)) + 1j * rng.normal(size=(V, 4))
        bd = torch.from_numpy(b).cuda()
        x_ctx = torch.zeros_like(bd)
        st_ctx = ctx.cg_solve(bd, x_ctx, mtype=mtype, tol=1e-12, tol_mode=yk.YK_TOL_REL)
        ctx.synchronize()
        want = x_ctx.cpu().numpy()
        stream = torch.cuda.current_stream().cuda_stream
        outs = [torch.full_like(bd, float("nan")) for _ in range(2)]   # every buffer allocated up front
        torch.cuda.synchronize()
        free = [torch.cuda.mem_get_info()[0]]
        for call in range(2):
            x = outs[call]
            st = yk.SolveStats()
            rc = yk.lib().yk_cg_solve_static(C.c_void_p(ctx.field_ptr()), Nt, Nx, a.m0, a.g, a.r,
                                             C.c_void_p(bd.data_ptr()), C.c_void_p(x.data_ptr()), mtype, 1e-12,
                                             yk.YK_TOL_REL, 1000, C.c_void_p(stream), C.byref(st))
            assert rc == yk.YK_OK, (call, yk.lib().yk_last_error())
            got = x.cpu().numpy()
            err = np.abs(got - want).max() / np.abs(want).max()
            assert err < 1e-12, (call, err)
            assert st.converged == 1 and st.iterations == st_ctx.iterations, (call, st.iterations)
            free.append(torch.cuda.mem_get_info()[0])
        # no device memory taken by the entry point: the second call leaves the
        # free memory exactly as the first left it; the first may only add the
        # library's fixed scratch array (about 6.6 MB), when the CUDA loader
        # brings its module in lazily at that call
        assert free[2] == free[1], free
        assert 0 <= free[0] - free[1] <= STATIC_BYTES_BOUND, free


def test_static_solve_refuses_large_lattice(ylib, cuda):
    yk, torch = ylib, cuda
    Nt, Nx = 256, 128          # 32768 sites > the 16384 of the static scratch
    sig = torch.zeros(Nt * Nx, dtype=torch.float64, device="cuda")
    b = torch.zeros(Nt * Nx * 4, dtype=torch.complex128, device="cuda")
    x = torch.zeros_like(b)
    rc = yk.lib().yk_cg_solve_static(C.c_void_p(sig.data_ptr()), Nt, Nx, 0.1, 0.5, 1.0, C.c_void_p(b.data_ptr()),
                                     C.c_void_p(x.data_ptr()), 1, 1e-8, yk.YK_TOL_ABS, 1000, None, None)
    assert rc == yk.YK_EINVAL
    assert b"static scratch" in yk.lib().yk_last_error()
