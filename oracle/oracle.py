"""ctypes wrapper of the CPU oracle (oracle/yukawa_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA path and the timed CPU
baseline.  Spinors are numpy complex128 arrays of shape (V, 4) (site-major,
[f1s1, f1s2, f2s1, f2s2]); fields are float64 arrays of shape (V,).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from .build_oracle import build

_lib = None


class Action(C.Structure):
    _fields_ = [("m2", C.c_double), ("lam", C.c_double), ("kappa", C.c_double), ("sq2kappa", C.c_double),
                ("g", C.c_double), ("m0", C.c_double), ("r", C.c_double), ("cut_fraction", C.c_double),
                ("eps_bar", C.c_double), ("drift_mode", C.c_int), ("use_mass", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        d, i, u32, u64, i64 = C.c_double, C.c_int, C.c_uint32, C.c_uint64, C.c_int64
        P = C.c_void_p
        A = C.POINTER(Action)
        sig = {
            "yko_derive": (None, [i, d, d, d, d, d, d, d, d, d, i, A]),
            "yko_dirac": (None, [i, i, A, P, P, P, i]),
            "yko_cg": (i, [i, i, A, P, P, P, i, d, i, i, C.POINTER(d)]),
            "yko_force": (i, [i, i, A, P, P, i, d, i, i, P]),
            "yko_mask_half": (None, [i, i, d, P]),
            "yko_mask_all_kept": (i, [i, i, d]),
            "yko_fft2": (None, [i, i, P, i]),
            "yko_coloured_noise": (None, [i, i, d, P, P]),
            "yko_bosonic_drift": (None, [i, i, d, d, P, P]),
            "yko_euler_update": (d, [i, d, d, P, P, P, C.POINTER(d)]),
            "yko_time_slices": (None, [i, i, P, P]),
            "yko_time_slices_spinor": (None, [i, i, P, P]),
            "yko_philox4x32_10": (None, [P, P, P]),
            "yko_normals": (None, [u64, u32, u64, u32, u32, i64, P]),
            "yko_normals_fp64": (None, [u64, u32, u64, u32, u32, i64, P]),
            "yko_normal_pair_words": (None, [u32, u32, P]),
            "yko_ff_ops": (None, [i64, P, P, P, P, P]),
            "yko_ff_hop": (None, [i, i, d, P, d, P, P, P, P, d, d, P]),
            "yko_uniform_field": (None, [u64, u32, i64, P]),
            "yko_uniform_field_comp": (None, [u64, u32, u32, i64, P]),
            "yko_drand48_field": (None, [i64, P]),
            "yko_langevin_step": (d, [i, i, A, u64, u32, u64, i, d, i, i, d, P, P]),
            "yko_gamma_method": (None, [P, i64, d, P]),
            "yko_dirac_pi": (None, [i, i, A, P, P, P, P, i]),
            "yko_cg_pi": (i, [i, i, A, P, P, P, P, i, d, i, i, C.POINTER(d)]),
            "yko_force_pi": (i, [i, i, A, P, P, P, i, d, i, i, P]),
            "yko_langevin_step_pi": (d, [i, i, A, u64, u32, u64, i, d, i, i, d, P, P]),
            "yko_threads": (i, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def derive(use_mass=0, mass=0.2, g_phys=0.0, kappa=0.18, lam=0.02, yukawa=1.0, fermion_mass=1.0, wilson=1.0,
           cut_fraction=1.0, average_epsilon=0.02, drift_mode=0) -> Action:
    """code/src/main.cu:58-63, 113-170"""
    a = Action()
    lib().yko_derive(int(use_mass), mass, g_phys, kappa, lam, yukawa, fermion_mass, wilson, cut_fraction,
                     average_epsilon, int(drift_mode), C.byref(a))
    return a


def action(m2=-0.5, lam=1.0, g=0.5, m0=0.1, r=1.0, cut_fraction=1.0, eps_bar=0.02, drift_mode=0) -> Action:
    """An action given directly in the kernels' units (useMass = "true")."""
    return derive(use_mass=1, mass=m2, g_phys=lam, yukawa=g, fermion_mass=m0, wilson=r, cut_fraction=cut_fraction,
                  average_epsilon=eps_bar, drift_mode=drift_mode)


def dirac(Nt, Nx, a: Action, sigma, psi, dagger=False):
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    psi = np.ascontiguousarray(psi, dtype=np.complex128).reshape(Nt * Nx, 4)
    out = np.empty_like(psi)
    lib().yko_dirac(Nt, Nx, C.byref(a), _p(sigma), _p(psi), _p(out), int(bool(dagger)))
    return out


def cg(Nt, Nx, a: Action, sigma, b, mtype=1, tol=1e-8, tol_mode=0, max_iter=1000):
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).reshape(Nt * Nx, 4)
    x = np.empty_like(b)
    rr = C.c_double()
    it = lib().yko_cg(Nt, Nx, C.byref(a), _p(sigma), _p(b), _p(x), int(mtype), tol, int(tol_mode), int(max_iter),
                      C.byref(rr))
    return x, it, rr.value


def force(Nt, Nx, a: Action, sigma, eta, tol=1e-8, tol_mode=0, max_iter=1000):
    """eta: (n_rhs, V, 4) complex"""
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    eta = np.ascontiguousarray(eta, dtype=np.complex128).reshape(-1, Nt * Nx, 4)
    F = np.empty(Nt * Nx)
    it = lib().yko_force(Nt, Nx, C.byref(a), _p(sigma), _p(eta), eta.shape[0], tol, int(tol_mode), int(max_iter),
                         _p(F))
    return F, it


def mask_half(Nt, Nx, cut_fraction):
    m = np.empty(Nt * (Nx // 2 + 1))
    lib().yko_mask_half(Nt, Nx, cut_fraction, _p(m))
    return m.reshape(Nt, Nx // 2 + 1)


def mask_all_kept(Nt, Nx, cut_fraction) -> bool:
    return bool(lib().yko_mask_all_kept(Nt, Nx, cut_fraction))


def fft2(Nt, Nx, z, sign=-1):
    z = np.ascontiguousarray(z, dtype=np.complex128).reshape(Nt, Nx).copy()
    lib().yko_fft2(Nt, Nx, _p(z), int(sign))
    return z


def coloured_noise(Nt, Nx, cut_fraction, white):
    white = np.ascontiguousarray(white, dtype=np.float64)
    xi = np.empty(Nt * Nx)
    lib().yko_coloured_noise(Nt, Nx, cut_fraction, _p(white), _p(xi))
    return xi


def bosonic_drift(Nt, Nx, m2, lam, phi, drift=None):
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    d = np.zeros(Nt * Nx) if drift is None else np.ascontiguousarray(drift, dtype=np.float64).copy()
    lib().yko_bosonic_drift(Nt, Nx, m2, lam, _p(phi), _p(d))
    return d


def euler_update(phi, drift, noise, eps_bar, fixed_dt=0.0):
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    drift = np.ascontiguousarray(drift, dtype=np.float64)
    noise = np.ascontiguousarray(noise, dtype=np.float64)
    m = C.c_double()
    eps = lib().yko_euler_update(phi.size, eps_bar, fixed_dt, _p(phi), _p(drift), _p(noise), C.byref(m))
    return phi, eps, m.value


def time_slices(Nt, Nx, phi):
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    out = np.empty(Nt)
    lib().yko_time_slices(Nt, Nx, _p(phi), _p(out))
    return out


def time_slices_spinor(Nt, Nx, psi):
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    out = np.empty(Nt)
    lib().yko_time_slices_spinor(Nt, Nx, _p(psi), _p(out))
    return out


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32).copy()
    k = np.asarray(key, dtype=np.uint32).copy()
    o = np.empty(4, dtype=np.uint32)
    lib().yko_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def normals(seed, chain, step, kind, rhs, n):
    """Normals 0 .. n-1 of Philox stream (seed, chain; step, kind, rhs): the
    FP32 Box-Muller of the CUDA generator, bit for bit."""
    out = np.empty(n)
    lib().yko_normals(seed, chain, step, kind, rhs, n, _p(out))
    return out


def normal_pair_words(a, b):
    """The generator's pair from explicit Philox words: a sets the radius, b the angle."""
    out = np.empty(2)
    lib().yko_normal_pair_words(a, b, _p(out))
    return out


def ff_ops(a, b):
    """The GPU even-odd kernels' float-float sum, product and reciprocal of the
    float-float splits of a and b (accuracy tests)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    s, p, r = np.empty_like(a), np.empty_like(a), np.empty_like(a)
    lib().yko_ff_ops(a.size, _p(a), _p(b), _p(s), _p(p), _p(r))
    return s, p, r


def ff_hop(dag, mode, r, c, diag, tu, td, xu, xd, sp, sm):
    """One real site of the kernels' float-float half hop (four components)."""
    arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (c, tu, td, xu, xd)]
    out = np.empty(4)
    lib().yko_ff_hop(int(dag), int(mode), float(r), _p(arrs[0]), float(diag), _p(arrs[1]), _p(arrs[2]),
                     _p(arrs[3]), _p(arrs[4]), float(sp), float(sm), _p(out))
    return out


def normals_fp64(seed, chain, step, kind, rhs, n):
    """The same Philox words through an FP64 libm Box-Muller."""
    out = np.empty(n)
    lib().yko_normals_fp64(seed, chain, step, kind, rhs, n, _p(out))
    return out


def uniform_field(seed, chain, n):
    out = np.empty(n)
    lib().yko_uniform_field(seed, chain, n, _p(out))
    return out


def uniform_pions(seed, chain, n):
    """The pion extension's initial pions (3, n): Philox uniform, comp 1..3."""
    out = np.empty((3, n))
    for a in range(3):
        lib().yko_uniform_field_comp(seed, chain, a + 1, n, _p(out[a]))
    return out


def drand48_field(n):
    out = np.empty(n)
    lib().yko_drand48_field(n, _p(out))
    return out


@dataclass
class StepObs:
    eps: float
    max_drift: float
    sum_phi: float
    sum_force: float
    cg_iters: int
    sum_phi2: float


def langevin_step(Nt, Nx, a: Action, phi, seed, chain, step, n_rhs=1, tol=1e-8, tol_mode=0, max_iter=1000,
                  fixed_dt=0.0):
    """One framework Langevin step; returns (new phi, StepObs)."""
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    obs = np.zeros(6)
    lib().yko_langevin_step(Nt, Nx, C.byref(a), seed, chain, step, n_rhs, tol, int(tol_mode), int(max_iter),
                            fixed_dt, _p(phi), _p(obs))
    return phi, StepObs(obs[0], obs[1], obs[2], obs[3], int(obs[4]), obs[5])


def gamma_method(data, stau=1.5):
    d = np.ascontiguousarray(data, dtype=np.float64)
    out = np.zeros(5)
    lib().yko_gamma_method(_p(d), d.size, stau, _p(out))
    return out


def fermion_eta(seed, chain, step, Nt, Nx, n_rhs=1, kind=2):
    """The framework's Philox fermion noise: real normals, imaginary parts 0."""
    V = Nt * Nx
    eta = np.zeros((n_rhs, V, 4), dtype=np.complex128)
    for j in range(n_rhs):
        eta[j].real = normals(seed, chain, step, kind, j, 4 * V).reshape(V, 4)
    return eta


def threads() -> int:
    return lib().yko_threads()


# ---------------------------------------------------------------- pion extension
def _pi(pi, V):
    if pi is None:
        return None, None
    a = np.ascontiguousarray(pi, dtype=np.float64).reshape(3 * V)
    return a, _p(a)


def dirac_pi(Nt, Nx, a: Action, sigma, pi, psi, dagger=False):
    """D with the Yukawa term g (sigma + i gamma5 tau.pi); pi: (3, V) or None."""
    V = Nt * Nx
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    psi = np.ascontiguousarray(psi, dtype=np.complex128).reshape(V, 4)
    keep, pp = _pi(pi, V)
    out = np.empty_like(psi)
    lib().yko_dirac_pi(Nt, Nx, C.byref(a), _p(sigma), pp, _p(psi), _p(out), int(bool(dagger)))
    return out


def cg_pi(Nt, Nx, a: Action, sigma, pi, b, mtype=1, tol=1e-8, tol_mode=0, max_iter=1000):
    V = Nt * Nx
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).reshape(V, 4)
    keep, pp = _pi(pi, V)
    x = np.empty_like(b)
    rr = C.c_double()
    it = lib().yko_cg_pi(Nt, Nx, C.byref(a), _p(sigma), pp, _p(b), _p(x), int(mtype), tol, int(tol_mode),
                         int(max_iter), C.byref(rr))
    return x, it, rr.value


def force_pi(Nt, Nx, a: Action, sigma, pi, eta, tol=1e-8, tol_mode=0, max_iter=1000):
    """eta: (n_rhs, V, 4) complex.  Returns F (4, V): sigma, pi1, pi2, pi3."""
    V = Nt * Nx
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    eta = np.ascontiguousarray(eta, dtype=np.complex128).reshape(-1, V, 4)
    keep, pp = _pi(pi, V)
    F = np.empty(4 * V)
    it = lib().yko_force_pi(Nt, Nx, C.byref(a), _p(sigma), pp, _p(eta), eta.shape[0], tol, int(tol_mode),
                            int(max_iter), _p(F))
    return F.reshape(4, V), it


@dataclass
class StepObsPi:
    eps: float
    max_drift: float
    sum_phi: float
    sum_force: float
    cg_iters: int
    sum_phi2: float
    sum_pi: tuple
    sum_pi2: float


def langevin_step_pi(Nt, Nx, a: Action, phi4, seed, chain, step, n_rhs=1, tol=1e-8, tol_mode=0, max_iter=1000,
                     fixed_dt=0.0):
    """One step of the four fields phi4 (4, V) = (sigma, pi1, pi2, pi3)."""
    phi4 = np.ascontiguousarray(phi4, dtype=np.float64).reshape(4 * Nt * Nx).copy()
    obs = np.zeros(10)
    lib().yko_langevin_step_pi(Nt, Nx, C.byref(a), seed, chain, step, n_rhs, tol, int(tol_mode), int(max_iter),
                               fixed_dt, _p(phi4), _p(obs))
    return phi4.reshape(4, Nt * Nx), StepObsPi(obs[0], obs[1], obs[2], obs[3], int(obs[4]), obs[5],
                                               (obs[6], obs[7], obs[8]), obs[9])
