"""GB300-native Langevin hot path of the 2-D Yukawa model (Matteo294/YukawaColouredNoise).

The product is the C-ABI library ``lib/libyukawa_gb300.so`` (include/yukawa.h);
this module binds it with ctypes and mirrors the reference's host classes so
that code written against the reference reads the same:

    reference (code/src/)                         here
    DiracOP<double>::applyD(in, out, MatrixType)  DiracOP(ctx).applyD(in, out, MatrixType.Normal)
    CGsolver::solve(in, out, D, MatrixType)       CGsolver(ctx).solve(in, out, D, MatrixType.Dagger)
    FermionicDrift::getForce(out, D, CG, ...)     FermionicDrift(ctx).getForce(out, D, CG)
    ColouredNoise::operator()()                   ColouredNoise(ctx)()
    ./out input.toml                              run("input.toml")   /  lib/yk_run input.toml

Device buffers are passed as objects with ``data_ptr()`` (torch tensors) or
raw integer addresses.  There is no CPU fallback: importing without the
built library raises.
"""
from __future__ import annotations

import ctypes as C
import enum
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libyukawa_gb300.so"

YK_OK, YK_EINVAL, YK_ENOCONV, YK_ENAN, YK_ETIMEOUT, YK_ECUDA, YK_ENOMEM, YK_EIO = range(8)
YK_NORMAL, YK_DAGGER = 0, 1
YK_FP64, YK_FP32, YK_MIXED = 0, 1, 2
YK_TOL_ABS, YK_TOL_REL = 0, 1
YK_INIT_DRAND48, YK_INIT_PHILOX, YK_INIT_NONE = 0, 1, 2


class MatrixType(enum.IntEnum):
    """code/src/params.h:8"""
    Normal = YK_NORMAL
    Dagger = YK_DAGGER


class YukawaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[status {status}] {msg}")
        self.status = status


class Params(C.Structure):
    """yk_params: input.toml keys + [lattice] + [gpu] extensions."""
    _fields_ = [
        ("use_mass", C.c_int), ("mass", C.c_double), ("g", C.c_double), ("kappa", C.c_double),
        ("lam", C.c_double), ("cut_fraction", C.c_double),
        ("average_epsilon", C.c_double), ("max_langevin_time", C.c_double), ("export_time", C.c_double),
        ("burn_count", C.c_int), ("measure_drift_count", C.c_int),
        ("seed", C.c_int64),
        ("yukawa_coupling", C.c_double), ("fermion_mass", C.c_double), ("drift_mode", C.c_int),
        ("wilson_param", C.c_double),
        ("Nt", C.c_int), ("Nx", C.c_int),
        ("precision", C.c_int), ("n_rhs", C.c_int), ("cg_tol_mode", C.c_int), ("cg_tol", C.c_double),
        ("cg_max_iter", C.c_int), ("reliable_every", C.c_int), ("reliable_delta", C.c_double),
        ("fixed_dt", C.c_double), ("init", C.c_int), ("learned_layers", C.c_int), ("pions", C.c_int),
    ]

    @classmethod
    def default(cls, **kw) -> "Params":
        p = cls()
        lib().yk_params_default(C.byref(p))
        for k, v in kw.items():
            if not hasattr(p, k):
                raise AttributeError(k)
            setattr(p, k, v)
        return p

    @classmethod
    def from_toml(cls, path) -> "Params":
        p = cls()
        _check(lib().yk_params_from_toml(str(path).encode(), C.byref(p)))
        return p

    def action(self) -> "Action":
        a = Action()
        _check(lib().yk_derive_action(C.byref(self), C.byref(a)))
        return a

    def copy(self, **kw) -> "Params":
        p = Params()
        C.pointer(p)[0] = self
        for k, v in kw.items():
            setattr(p, k, v)
        return p


class Action(C.Structure):
    _fields_ = [("m2", C.c_double), ("lam", C.c_double), ("kappa", C.c_double), ("sq2kappa", C.c_double),
                ("g", C.c_double), ("m0", C.c_double), ("r", C.c_double), ("cut_fraction", C.c_double),
                ("eps_bar", C.c_double), ("drift_mode", C.c_int), ("use_mass", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("reliable_updates", C.c_int), ("rr", C.c_double),
                ("rr0", C.c_double), ("converged", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("cg_grid", C.c_int), ("cg_grid_max", C.c_int), ("cg_candidates", C.c_int),
                ("cg_ms_chosen", C.c_float), ("cg_ms_max", C.c_float), ("conv_rows", C.c_int),
                ("conv_cols", C.c_int), ("conv_layers_per_launch", C.c_int), ("pcg_inner_tol", C.c_double),
                ("noise_overlap", C.c_int), ("step_ms_overlap", C.c_float), ("step_ms_serial", C.c_float)]


class NetTrainCfg(C.Structure):
    _fields_ = [("n_sources", C.c_int), ("n_levels", C.c_int), ("base_iter", C.c_int), ("steps", C.c_int),
                ("batch", C.c_int), ("lr", C.c_double), ("seed", C.c_uint64)]


class NetTrainStats(C.Structure):
    _fields_ = [("pairs", C.c_int), ("loss0", C.c_double), ("loss1", C.c_double), ("ms", C.c_double)]


class Obs(C.Structure):
    _fields_ = [("t", C.c_double), ("eps", C.c_double), ("max_drift", C.c_double), ("sum_phi", C.c_double),
                ("sum_phi2", C.c_double), ("sum_force", C.c_double), ("steps", C.c_int64),
                ("cg_iterations", C.c_int), ("cg_iterations_total", C.c_int64), ("noconv_steps", C.c_int64),
                ("status", C.c_int), ("sum_pi", C.c_double * 3), ("sum_pi2", C.c_double)]


class SeriesStats(C.Structure):
    """yk_series_stats: each field {value, error, error of error, tau_int, tau_int error}."""
    _fields_ = [("n", C.c_int64), ("sigma", C.c_double * 5), ("abs_sigma", C.c_double * 5),
                ("chi", C.c_double * 5), ("binder", C.c_double * 5)]

    def as_dict(self):
        return {k: list(getattr(self, k)) for k in ("sigma", "abs_sigma", "chi", "binder")} | {"n": self.n}


class Profile(C.Structure):
    _fields_ = [("steps", C.c_int), ("launches", C.c_int), ("cg_launches", C.c_int), ("cg_grid", C.c_int),
                ("cg_kernel", C.c_int),
                ("noise_ms", C.c_double), ("cg_ms", C.c_double), ("force_ms", C.c_double),
                ("update_ms", C.c_double), ("cg_iterations", C.c_int64), ("cg_site_iterations", C.c_int64),
                ("sites", C.c_int64)]


_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "yk_last_error": (C.c_char_p, []),
    "yk_version": (C.c_char_p, []),
    "yk_params_default": (None, [C.POINTER(Params)]),
    "yk_params_from_toml": (C.c_int, [C.c_char_p, C.POINTER(Params)]),
    "yk_derive_action": (C.c_int, [C.POINTER(Params), C.POINTER(Action)]),
    "yk_ctx_create": (C.c_int, [C.POINTER(Params), C.c_int, C.POINTER(C.c_void_p)]),
    "yk_ctx_destroy": (C.c_int, [C.c_void_p]),
    "yk_ctx_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "yk_ctx_synchronize": (C.c_int, [C.c_void_p]),
    "yk_ctx_n_chains": (C.c_int, [C.c_void_p]),
    "yk_ctx_volume": (C.c_int, [C.c_void_p, C.c_int]),
    "yk_ctx_shape": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "yk_set_field_host": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "yk_get_field_host": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "yk_field_device": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "yk_set_pions_host": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "yk_get_pions_host": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "yk_pions_device": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "yk_dirac_apply": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "yk_cg_solve": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int,
                              C.c_int, C.c_int, C.POINTER(SolveStats)]),
    "yk_cg_solve_static": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_void_p,
                                     C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int, C.c_void_p,
                                     C.POINTER(SolveStats)]),
    "yk_check_wait_timeout": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "yk_net_setup": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_uint64, C.c_double]),
    "yk_net_size": (C.c_int, [C.c_void_p, C.c_int]),
    "yk_net_weights": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "yk_net_apply": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "yk_net_apply_tc": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "yk_net_grad": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "yk_net_train": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(NetTrainCfg), C.POINTER(NetTrainStats)]),
    "yk_fgcr_solve": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int,
                                C.POINTER(SolveStats)]),
    "yk_autotune": (C.c_int, [C.c_void_p, C.POINTER(TuneResult)]),
    "yk_tune_report": (C.c_int, [C.c_void_p, C.POINTER(TuneResult)]),
    "yk_langevin_step_learned": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(SolveStats)]),
    "yk_pcg_solve": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int,
                               C.POINTER(SolveStats)]),
    "yk_fermion_force": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(SolveStats)]),
    "yk_coloured_noise": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "yk_langevin_step": (C.c_int, [C.c_void_p, C.c_int]),
    "yk_langevin_step_io": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "yk_euler_update": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(Obs)]),
    "yk_observables": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Obs)]),
    "yk_profile_begin": (C.c_int, [C.c_void_p]),
    "yk_profile_end": (C.c_int, [C.c_void_p, C.POINTER(Profile)]),
    "yk_time_slices": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "yk_correlator": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(SolveStats)]),
    "yk_condensate": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(SolveStats)]),
    "yk_set_eps_bar": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "yk_get_step": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int64)]),
    "yk_set_step": (C.c_int, [C.c_void_p, C.c_int, C.c_int64]),
    "yk_set_time": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "yk_checkpoint_save": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_double]),
    "yk_checkpoint_load": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.POINTER(C.c_double)]),
    "yk_gamma_method": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.c_void_p]),
    "yk_run_toml": (C.c_int, [C.c_char_p, C.c_char_p]),
    "yk_series_record": (C.c_int, [C.c_void_p, C.c_int, C.c_int64]),
    "yk_series_read": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "yk_series_analyse": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.POINTER(SeriesStats)]),
    "yk_series_analyse_host": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_double, C.POINTER(SeriesStats)]),
}


def lib():
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        _lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def exported_symbols():
    return list(_SIGS)


def _check(rc: int, ok=(YK_OK,)):
    if rc not in ok:
        raise YukawaError(rc, lib().yk_last_error().decode())
    return rc


def _ptr(buf) -> int:
    if buf is None:
        return None
    if isinstance(buf, int):
        return buf
    if hasattr(buf, "data_ptr"):
        return buf.data_ptr()
    raise TypeError(f"expected a device buffer (data_ptr()) or an address, got {type(buf)}")


class Context:
    """yk_ctx: one or more independent chains on the current CUDA device."""

    def __init__(self, params, n_chains: int | None = None):
        if isinstance(params, Params):
            params = [params] * (n_chains or 1)
        arr = (Params * len(params))(*params)
        h = C.c_void_p()
        _check(lib().yk_ctx_create(arr, len(params), C.byref(h)))
        self.h = h
        self.params = list(params)

    def close(self):
        if self.h:
            lib().yk_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def n_chains(self) -> int:
        return lib().yk_ctx_n_chains(self.h)

    def volume(self, chain=0) -> int:
        return lib().yk_ctx_volume(self.h, chain)

    def shape(self, chain=0):
        nt, nx = C.c_int(), C.c_int()
        _check(lib().yk_ctx_shape(self.h, chain, C.byref(nt), C.byref(nx)))
        return nt.value, nx.value

    def set_stream(self, stream_handle: int):
        _check(lib().yk_ctx_set_stream(self.h, C.c_void_p(stream_handle)))

    def synchronize(self):
        _check(lib().yk_ctx_synchronize(self.h))

    def set_field(self, phi, chain=0):
        import numpy as np
        a = np.ascontiguousarray(phi, dtype=np.float64)
        assert a.size == self.volume(chain)
        _check(lib().yk_set_field_host(self.h, chain, a.ctypes.data_as(C.c_void_p)))

    def get_field(self, chain=0):
        import numpy as np
        a = np.empty(self.volume(chain))
        _check(lib().yk_get_field_host(self.h, chain, a.ctypes.data_as(C.c_void_p)))
        return a

    def set_pions(self, pi, chain=0):
        """Pion extension: the chain's pi_1..3, shape (3, V)."""
        import numpy as np
        a = np.ascontiguousarray(pi, dtype=np.float64)
        assert a.size == 3 * self.volume(chain)
        _check(lib().yk_set_pions_host(self.h, chain, a.ctypes.data_as(C.c_void_p)))

    def get_pions(self, chain=0):
        import numpy as np
        a = np.empty(3 * self.volume(chain))
        _check(lib().yk_get_pions_host(self.h, chain, a.ctypes.data_as(C.c_void_p)))
        return a.reshape(3, -1)

    def pions_ptr(self, chain=0) -> int:
        p = C.c_void_p()
        _check(lib().yk_pions_device(self.h, chain, C.byref(p)))
        return p.value

    def field_ptr(self, chain=0) -> int:
        p = C.c_void_p()
        _check(lib().yk_field_device(self.h, chain, C.byref(p)))
        return p.value

    def dirac_apply(self, inp, out, dagger=False, precision=YK_FP64, chain=0):
        _check(lib().yk_dirac_apply(self.h, chain, _ptr(inp), _ptr(out), int(bool(dagger)), precision))

    def cg_solve(self, b, x, mtype=YK_DAGGER, tol=1e-8, tol_mode=YK_TOL_ABS, max_iter=1000, precision=YK_FP64,
                 chain=0, allow_noconv=False) -> SolveStats:
        st = SolveStats()
        ok = (YK_OK, YK_ENOCONV) if allow_noconv else (YK_OK,)
        _check(lib().yk_cg_solve(self.h, chain, _ptr(b), _ptr(x), int(mtype), tol, tol_mode, max_iter, precision,
                                 C.byref(st)), ok)
        return st

    # ---- learned preconditioner ----
    def net_setup(self, layers=4, seed=1, skip=-1.0, chain=0):
        _check(lib().yk_net_setup(self.h, chain, layers, seed, skip))

    def net_size(self, chain=0) -> int:
        return lib().yk_net_size(self.h, chain)

    def net_get_weights(self, chain=0):
        import numpy as np
        w = np.empty(self.net_size(chain), dtype=np.float32)
        _check(lib().yk_net_weights(self.h, chain, w.ctypes.data, 0))
        return w

    def net_set_weights(self, w, chain=0):
        import numpy as np
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.net_size(chain)
        _check(lib().yk_net_weights(self.h, chain, w.ctypes.data, 1))

    def net_apply(self, r, z, chain=0, tensor_cores=False):
        fn = lib().yk_net_apply_tc if tensor_cores else lib().yk_net_apply
        _check(fn(self.h, chain, _ptr(r), _ptr(z)))

    def net_grad(self, r, e, chain=0):
        import numpy as np
        g = np.empty(self.net_size(chain), dtype=np.float32)
        loss = C.c_double()
        _check(lib().yk_net_grad(self.h, chain, _ptr(r), _ptr(e), g.ctypes.data, C.byref(loss)))
        return g, loss.value

    def net_train(self, n_sources=4, n_levels=4, base_iter=4, steps=200, batch=4, lr=1e-3, seed=1,
                  chain=0) -> NetTrainStats:
        cfg = NetTrainCfg(n_sources, n_levels, base_iter, steps, batch, lr, seed)
        st = NetTrainStats()
        _check(lib().yk_net_train(self.h, chain, C.byref(cfg), C.byref(st)))
        return st

    def fgcr_solve(self, b, x, tol=1e-10, tol_mode=YK_TOL_REL, max_iter=2000, use_net=True, chain=0,
                   allow_noconv=False) -> SolveStats:
        st = SolveStats()
        ok = (YK_OK, YK_ENOCONV) if allow_noconv else (YK_OK,)
        _check(lib().yk_fgcr_solve(self.h, chain, _ptr(b), _ptr(x), tol, tol_mode, max_iter, int(bool(use_net)),
                                   C.byref(st)), ok)
        return st

    def pcg_solve(self, b, x, tol=1e-10, tol_mode=YK_TOL_REL, max_iter=2000, use_net=True, chain=0,
                  allow_noconv=False) -> SolveStats:
        st = SolveStats()
        ok = (YK_OK, YK_ENOCONV) if allow_noconv else (YK_OK,)
        _check(lib().yk_pcg_solve(self.h, chain, _ptr(b), _ptr(x), tol, tol_mode, max_iter, int(bool(use_net)),
                                  C.byref(st)), ok)
        return st

    def fermion_force(self, F, eta=None, chain=0) -> SolveStats:
        st = SolveStats()
        _check(lib().yk_fermion_force(self.h, chain, _ptr(eta), _ptr(F), C.byref(st)))
        return st

    def coloured_noise(self, xi, white=None, chain=0):
        _check(lib().yk_coloured_noise(self.h, chain, _ptr(white), _ptr(xi)))

    def step(self, n=1):
        _check(lib().yk_langevin_step(self.h, n))

    def step_io(self, phi_in=None, phi_out=None, chain=0) -> "Obs":
        """One step with chain `chain`'s field uploaded from and downloaded to
        host arrays (numpy float64 or pinned torch tensors; None: skipped) and
        its observables returned, one synchronisation."""
        import numpy as np
        V = self.volume(chain)

        def host(a, writable):
            if a is None:
                return None
            if isinstance(a, np.ndarray):
                if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or (writable and not a.flags["WRITEABLE"]):
                    raise TypeError("step_io: host arrays must be C-contiguous float64 (and writable for phi_out)")
                if a.size != V:
                    raise ValueError(f"step_io: {a.size} values for a lattice of {V} sites")
                return a.ctypes.data
            return _ptr(a)

        o = Obs()
        _check(lib().yk_langevin_step_io(self.h, chain, host(phi_in, False), host(phi_out, True), C.byref(o)))
        return o

    def autotune(self) -> TuneResult:
        t = TuneResult()
        _check(lib().yk_autotune(self.h, C.byref(t)))
        return t

    def tune_report(self) -> TuneResult:
        t = TuneResult()
        _check(lib().yk_tune_report(self.h, C.byref(t)))
        return t

    def step_learned(self, n=1, use_net=True) -> SolveStats:
        st = SolveStats()
        _check(lib().yk_langevin_step_learned(self.h, n, int(bool(use_net)), C.byref(st)))
        return st

    def euler_update(self, force, xi, chain=0) -> Obs:
        o = Obs()
        _check(lib().yk_euler_update(self.h, chain, _ptr(force), _ptr(xi), C.byref(o)))
        return o

    def profile_begin(self):
        _check(lib().yk_profile_begin(self.h))

    def profile_end(self) -> Profile:
        pr = Profile()
        _check(lib().yk_profile_end(self.h, C.byref(pr)))
        return pr

    def observables(self, chain=0) -> Obs:
        o = Obs()
        _check(lib().yk_observables(self.h, chain, C.byref(o)))
        return o

    def time_slices(self, chain=0):
        import numpy as np
        nt, _ = self.shape(chain)
        out = np.empty(nt)
        _check(lib().yk_time_slices(self.h, chain, out.ctypes.data_as(C.c_void_p)))
        return out

    def correlator(self, chain=0):
        import numpy as np
        nt, _ = self.shape(chain)
        out = np.empty(nt)
        st = SolveStats()
        _check(lib().yk_correlator(self.h, chain, out.ctypes.data_as(C.c_void_p), C.byref(st)))
        return out, st

    def condensate(self, chain=0):
        v = C.c_double()
        st = SolveStats()
        _check(lib().yk_condensate(self.h, chain, C.byref(v), C.byref(st)))
        return v.value, st

    def set_eps_bar(self, eps_bar, chain=0):
        _check(lib().yk_set_eps_bar(self.h, chain, eps_bar))

    def get_step(self, chain=0) -> int:
        v = C.c_int64()
        _check(lib().yk_get_step(self.h, chain, C.byref(v)))
        return v.value

    def set_step(self, step, chain=0):
        _check(lib().yk_set_step(self.h, chain, step))

    def series_record(self, capacity, chain=0):
        """Record <sigma> after every step on the device (capacity 0 stops)."""
        _check(lib().yk_series_record(self.h, chain, int(capacity)))

    def series_read(self, chain=0):
        import numpy as np
        n = C.c_int64()
        _check(lib().yk_series_read(self.h, chain, None, 0, C.byref(n)))
        have = C.c_int64()
        buf = np.empty(max(1, n.value))
        _check(lib().yk_series_read(self.h, chain, buf.ctypes.data_as(C.c_void_p), buf.size, C.byref(have)))
        return buf[:have.value].copy()

    def series_analyse(self, stau=1.5, chain=0) -> SeriesStats:
        st = SeriesStats()
        _check(lib().yk_series_analyse(self.h, chain, stau, C.byref(st)))
        return st

    def checkpoint_save(self, path, eps_bar, chain=0):
        _check(lib().yk_checkpoint_save(self.h, chain, str(path).encode(), eps_bar))

    def checkpoint_load(self, path, chain=0) -> float:
        e = C.c_double()
        _check(lib().yk_checkpoint_load(self.h, chain, str(path).encode(), C.byref(e)))
        return e.value


# ---------------------------------------------------------------------------
# Mirrors of the reference's host classes (code/src/*.cuh).
# ---------------------------------------------------------------------------
class DiracOP:
    """DiracOP<double> (code/src/Dirac.cuh:16-27); sigma is the chain's field."""

    def __init__(self, ctx: Context, chain=0):
        self.ctx, self.chain = ctx, chain

    def applyD(self, inp, out, MType=MatrixType.Normal, precision=YK_FP64):
        self.ctx.dirac_apply(inp, out, MType == MatrixType.Dagger, precision, self.chain)


class CGsolver:
    """CGsolver (code/src/CGsolver.cuh:32-53); tolerance and IterMax default to params.h:13-15."""

    def __init__(self, ctx: Context, chain=0, tol=1e-8, tol_mode=YK_TOL_ABS, max_iter=1000, precision=YK_FP64):
        self.ctx, self.chain = ctx, chain
        self.tol, self.tol_mode, self.max_iter, self.precision = tol, tol_mode, max_iter, precision
        self.last = None

    def solve(self, inVec, outVec, D: DiracOP | None = None, Mtype=MatrixType.Dagger) -> SolveStats:
        self.last = self.ctx.cg_solve(inVec, outVec, int(Mtype), self.tol, self.tol_mode, self.max_iter,
                                      self.precision, self.chain, allow_noconv=True)
        return self.last


class FermionicDrift:
    """FermionicDrift (code/src/FermionicDrift.cuh:11-32): Philox noise instead of per-element XORWOW states."""

    def __init__(self, ctx: Context, chain=0):
        self.ctx, self.chain = ctx, chain

    def getForce(self, outVec, D: DiracOP | None = None, CG: CGsolver | None = None, eta=None) -> SolveStats:
        return self.ctx.fermion_force(outVec, eta, self.chain)


class ColouredNoise:
    """ColouredNoise (code/src/colouredNoise.h:26-51): xi = filtered white noise."""

    def __init__(self, ctx: Context, noise, chain=0):
        self.ctx, self.noise, self.chain = ctx, noise, chain

    def __call__(self, white=None):
        self.ctx.coloured_noise(self.noise, white, self.chain)


def gamma_method(data, stau=1.5):
    """Wolff Gamma-method: (mean, error, error of error, tau_int, tau_int error)."""
    import numpy as np
    d = np.ascontiguousarray(data, dtype=np.float64)
    out = np.zeros(5)
    _check(lib().yk_gamma_method(d.ctypes.data_as(C.c_void_p), d.size, stau, out.ctypes.data_as(C.c_void_p)))
    return tuple(out)


def series_stats(series, volume, stau=1.5) -> SeriesStats:
    """yk_series_analyse_host: <sigma>, <|sigma|>, chi, Binder with Gamma-method errors (GPU)."""
    import numpy as np
    a = np.ascontiguousarray(series, dtype=np.float64)
    st = SeriesStats()
    _check(lib().yk_series_analyse_host(a.ctypes.data_as(C.c_void_p), a.size, int(volume), stau, C.byref(st)))
    return st


def run(toml_path, out_dir="."):
    """The reference's `./out input.toml` protocol (main.cu:73-516)."""
    _check(lib().yk_run_toml(str(toml_path).encode(), str(out_dir).encode()))
