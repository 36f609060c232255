"""ctypes binding of the engine's C ABI (include/lqg.h).

The engine is the compiled library lyspeq_gb300/liblqg.so; there is no
fallback: if the library is missing or a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# LQG_LIB selects another build of the same ABI (e.g. liblqg_checked.so)
LIB_PATH = os.environ.get("LQG_LIB", os.path.join(HERE, "liblqg.so"))

LQG_OK = 0
PRECISION = {"fp64": 0, "mixed": 1, "mixed_direct": 2, "mixed_auto": 3}
TUNING_FIELDS = 5   # LQG_TUNING_FIELDS: ld, form, drain, Gram K per split, CTA pairs
CHUNK_STATUS = {0: "ok", 1: "short", 2: "no_table", 3: "empty", 4: "out_of_range",
                5: "not_spd", 6: "bad_input", 7: "too_large", 8: "timeout", 9: "index_check"}

EXPORTS = ["lqg_abi_version", "lqg_ctx_create", "lqg_ctx_destroy", "lqg_last_error",
           "lqg_batch_add", "lqg_batch_clear", "lqg_batch_size", "lqg_chunk_info",
           "lqg_nr_iteration", "lqg_download", "lqg_chunk_result", "lqg_fisher_solve",
           "lqg_last_timings", "lqg_last_launch_count", "lqg_last_wave_count", "lqg_batch_add_reso",
           "lqg_resomat_deconvolve", "lqg_resomat_oversample", "lqg_tables_generate",
           "lqg_bootstrap", "lqg_smooth_ivar", "lqg_bootstrap_complete", "lqg_bootstrap_coefficients",
           "lqg_resomat_smooth", "lqg_fisher_solve_n", "lqg_set_wait_limit", "lqg_factor_noalloc",
           "lqg_probe_fp64_rate", "lqg_nr_iteration_async", "lqg_sync", "lqg_autotune", "lqg_tuning_get",
           "lqg_tuning_set", "lqg_set_fisher_optimization", "lqg_chunk_plan", "lqg_last_h2d_bytes"]


class LqgBins(C.Structure):
    _fields_ = [("nk", C.c_int), ("nz", C.c_int), ("k_edges", C.POINTER(C.c_double)),
                ("z_centers", C.POINTER(C.c_double)), ("z_bin_width", C.c_double),
                ("triangular", C.c_int)]


class LqgTables(C.Structure):
    _fields_ = [("n_tables", C.c_int), ("r_fwhm", C.POINTER(C.c_int)),
                ("dv", C.POINTER(C.c_double)), ("nv", C.c_int), ("v_length", C.c_double),
                ("nzp", C.c_int), ("deriv", C.POINTER(C.c_double)),
                ("signal", C.POINTER(C.c_double))]


class LqgOpts(C.Structure):
    _fields_ = [("max_forest_length", C.c_double), ("max_mean_pixel_size", C.c_double),
                ("cont_logl_order", C.c_int), ("cont_l_order", C.c_int),
                ("turn_off_sfid", C.c_int), ("skip_fisher", C.c_int),
                ("workspace_bytes", C.c_size_t), ("smooth_noise_weights", C.c_int),
                ("redshift_growth_on", C.c_int), ("fid_redshift_power", C.c_double)]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load liblqg.so and declare the signatures; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built: run `python -m lyspeq_gb300.build`")
    lib = C.CDLL(path)
    dp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p
    lib.lqg_abi_version.restype = C.c_int
    lib.lqg_ctx_create.argtypes = [C.POINTER(vp), C.POINTER(LqgBins), C.POINTER(LqgTables),
                                   C.POINTER(LqgOpts), C.c_int]
    lib.lqg_ctx_destroy.argtypes = [vp]
    lib.lqg_last_error.argtypes = [vp]
    lib.lqg_last_error.restype = C.c_char_p
    lib.lqg_batch_add.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), dp, dp, dp, ip, ip]
    lib.lqg_batch_add_reso.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), dp, dp, dp, C.c_int, C.c_int,
                                       dp, ip]
    lib.lqg_resomat_deconvolve.argtypes = [C.c_int, C.c_int, dp, C.c_double]
    lib.lqg_resomat_oversample.argtypes = [C.c_int, C.c_int, dp, C.c_int, C.c_double, dp]
    lib.lqg_tables_generate.argtypes = [C.POINTER(LqgBins), C.c_int, ip, dp, C.c_int, C.c_double, C.c_int,
                                        dp, C.c_int, dp, dp, C.c_int]
    lib.lqg_bootstrap.argtypes = [vp, C.c_int, ip, C.c_int, C.c_ulonglong, dp, dp, dp, dp, dp]
    lib.lqg_smooth_ivar.argtypes = [C.c_int, dp, C.c_int, dp]
    lib.lqg_resomat_smooth.argtypes = [C.c_int, C.c_int, dp, C.c_int]
    lib.lqg_bootstrap_complete.argtypes = [vp, C.c_int, ip, C.c_int, C.c_ulonglong, dp, dp, dp, ip]
    lib.lqg_bootstrap_coefficients.argtypes = [C.c_int, C.c_int, C.c_ulonglong, C.c_int,
                                               C.POINTER(C.c_ubyte)]
    lib.lqg_batch_clear.argtypes = [vp]
    lib.lqg_batch_size.argtypes = [vp]
    lib.lqg_abi_version.argtypes = []
    lib.lqg_last_h2d_bytes.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.lqg_chunk_info.argtypes = [vp, C.c_int, ip]
    lib.lqg_chunk_plan.argtypes = [C.POINTER(LqgBins), C.POINTER(LqgTables), C.POINTER(LqgOpts), C.c_int,
                                   C.POINTER(C.c_int64), dp, dp, dp, ip, C.c_int, C.c_int, dp, ip, ip]
    lib.lqg_nr_iteration.argtypes = [vp, dp, C.c_int]
    lib.lqg_download.argtypes = [vp, dp, dp, dp, dp, ip]
    lib.lqg_chunk_result.argtypes = [vp, C.c_int, dp, dp, dp, dp]
    lib.lqg_fisher_solve.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, ip, ip, dp]
    lib.lqg_fisher_solve_n.argtypes = [C.c_int, dp, dp, dp, dp, dp, dp, dp, ip, ip, dp]
    lib.lqg_last_timings.argtypes = [vp, dp, C.c_int]
    lib.lqg_last_launch_count.argtypes = [vp]
    lib.lqg_last_wave_count.argtypes = [vp]
    lib.lqg_set_wait_limit.argtypes = [vp, C.c_double]
    lib.lqg_set_fisher_optimization.argtypes = [vp, C.c_int]
    lib.lqg_factor_noalloc.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, C.c_int, C.c_int, vp, vp, vp]
    lib.lqg_probe_fp64_rate.argtypes = [C.c_int, dp]
    lib.lqg_nr_iteration_async.argtypes = [vp, dp, C.c_int, vp]
    lib.lqg_sync.argtypes = [vp]
    lib.lqg_autotune.argtypes = [vp, C.c_double, C.c_int, C.c_int]
    lib.lqg_tuning_get.argtypes = [vp, ip, C.c_int]
    lib.lqg_tuning_set.argtypes = [vp, ip, C.c_int]
    _lib = lib
    return lib


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


class Engine:
    """One engine context on one GPU: the lookup tables, the binning and a
    batch of chunks (Chunk objects of the reference, kept on the device)."""

    def __init__(self, bins, tables, nv, lenv, nzp, max_forest_length, max_mean_pixel_size=150.0,
                 cont=(-1, -1), turn_off_sfid=False, skip_fisher=False, device=0,
                 workspace_bytes=0, smooth_noise_weights=-1, redshift_growth=False, fid_b=0.0):
        self.lib = load_library()
        self.bins = bins
        self.nkz = bins.nk * bins.nz
        self._k_edges = np.ascontiguousarray(bins.k_edges, dtype=np.float64)
        self._z = np.ascontiguousarray(bins.z_centers, dtype=np.float64)
        self._r = np.ascontiguousarray([t.r_fwhm for t in tables], dtype=np.int32)
        self._dv = np.ascontiguousarray([t.dv for t in tables], dtype=np.float64)
        self._deriv = np.ascontiguousarray(np.stack([t.deriv for t in tables]), dtype=np.float64)
        self._signal = np.ascontiguousarray(np.stack([t.signal for t in tables]), dtype=np.float64)
        b = LqgBins(bins.nk, bins.nz, _dptr(self._k_edges), _dptr(self._z), bins.dz,
                    1 if bins.triangular else 0)
        t = LqgTables(len(tables), _iptr(self._r), _dptr(self._dv), nv, lenv, nzp,
                      _dptr(self._deriv), None if turn_off_sfid else _dptr(self._signal))
        o = LqgOpts(max_forest_length, max_mean_pixel_size, cont[0], cont[1], int(turn_off_sfid),
                    int(skip_fisher), workspace_bytes, int(smooth_noise_weights), int(bool(redshift_growth)),
                    float(fid_b))
        h = C.c_void_p()
        rc = self.lib.lqg_ctx_create(C.byref(h), C.byref(b), C.byref(t), C.byref(o), device)
        if rc != LQG_OK:
            raise RuntimeError(f"lqg_ctx_create failed with {rc}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.lqg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != LQG_OK:
            raise RuntimeError(f"{what} failed ({rc}): {self.lib.lqg_last_error(self.h).decode()}")

    @staticmethod
    def _pixel_arrays(lam, delta, ivar, offsets):
        """The concatenated pixel arrays and chunk offsets as the C ABI reads
        them, checked here: it takes plain pointers and cannot."""
        lam = np.ascontiguousarray(lam, dtype=np.float64).ravel()
        delta = np.ascontiguousarray(delta, dtype=np.float64).ravel()
        ivar = np.ascontiguousarray(ivar, dtype=np.float64).ravel()
        offsets = np.ascontiguousarray(offsets, dtype=np.int64).ravel()
        if not (len(lam) == len(delta) == len(ivar)):
            raise ValueError("lambda, delta and ivar differ in length")
        if len(offsets) < 1 or offsets[0] < 0 or offsets[-1] > len(lam) or np.any(np.diff(offsets) < 0):
            raise ValueError("offsets must rise from >= 0 to at most the number of pixels")
        return lam, delta, ivar, offsets

    def add_chunks(self, lam, delta, ivar, offsets, r_fwhm):
        """Add chunks given as concatenated arrays; returns the per-chunk status."""
        lam, delta, ivar, offsets = self._pixel_arrays(lam, delta, ivar, offsets)
        r_fwhm = np.ascontiguousarray(r_fwhm, dtype=np.int32).ravel()
        n = len(offsets) - 1
        if len(r_fwhm) != n:
            raise ValueError("one r_fwhm per chunk")
        status = np.zeros(max(n, 1), dtype=np.int32)
        rc = self.lib.lqg_batch_add(self.h, n, offsets.ctypes.data_as(C.POINTER(C.c_int64)),
                                    _dptr(lam), _dptr(delta), _dptr(ivar), _iptr(r_fwhm),
                                    _iptr(status))
        self._check(rc, "lqg_batch_add")
        return status[:n]

    def add_chunk_list(self, chunks):
        """chunks: iterable of (lambda_angstrom, delta, ivar, r_fwhm)."""
        chunks = list(chunks)
        offs = np.zeros(len(chunks) + 1, dtype=np.int64)
        for i, c in enumerate(chunks):
            offs[i + 1] = offs[i] + len(c[0])
        cat = lambda j: np.concatenate([np.asarray(c[j], dtype=np.float64) for c in chunks]) \
            if chunks else np.zeros(0)
        return self.add_chunks(cat(0), cat(1), cat(2), offs, [c[3] for c in chunks])

    def add_chunks_reso(self, lam, delta, ivar, offsets, oversampling, resomat):
        """Add chunks with resolution matrices: resomat has one row of nelem
        values per pixel (see lqg_batch_add_reso); returns the per-chunk status."""
        lam, delta, ivar, offsets = self._pixel_arrays(lam, delta, ivar, offsets)
        rm = np.ascontiguousarray(resomat, dtype=np.float64)
        if rm.ndim != 2 or rm.shape[0] != len(lam):
            raise ValueError("resomat must have one row per pixel")
        n = len(offsets) - 1
        status = np.zeros(max(n, 1), dtype=np.int32)
        rc = self.lib.lqg_batch_add_reso(self.h, n, offsets.ctypes.data_as(C.POINTER(C.c_int64)),
                                         _dptr(lam), _dptr(delta), _dptr(ivar), int(oversampling),
                                         rm.shape[1], _dptr(rm), _iptr(status))
        self._check(rc, "lqg_batch_add_reso")
        return status[:n]

    def add_chunk_list_reso(self, chunks, oversampling):
        """chunks: iterable of (lambda_angstrom, delta, ivar, resomat), resomat
        the chunk's oversampled rows [n][nelem] (oversampling > 0) or its
        diagonal matrix values[ndiags][n] (oversampling <= 0)."""
        chunks = list(chunks)
        offs = np.zeros(len(chunks) + 1, dtype=np.int64)
        for i, c in enumerate(chunks):
            offs[i + 1] = offs[i] + len(c[0])
        cat = lambda j: np.concatenate([np.asarray(c[j], dtype=np.float64) for c in chunks])
        per_pixel = [np.asarray(c[3]) if oversampling > 0 else np.asarray(c[3]).T for c in chunks]
        return self.add_chunks_reso(cat(0), cat(1), cat(2), offs, oversampling, np.concatenate(per_pixel))

    def bootstrap(self, qso_offsets, nboots, seed=0, solver=None, realizations=False):
        """FastBootstrap over spectra (lqg_bootstrap): returns mean, fisher_cov
        (covariance / 4), cov (sandwiched with solver, if given) and optionally
        the realizations."""
        off = np.ascontiguousarray(qso_offsets, dtype=np.int32)
        nkz = self.nkz
        mean = np.zeros(nkz)
        fcov = np.zeros((nkz, nkz))
        cov = np.zeros((nkz, nkz)) if solver is not None else None
        real = np.zeros((nboots, nkz)) if realizations else None
        sv = None if solver is None else np.ascontiguousarray(solver, dtype=np.float64)
        if sv is not None and sv.shape != (nkz, nkz):
            raise ValueError(f"solver must be {nkz} x {nkz}")
        rc = self.lib.lqg_bootstrap(self.h, len(off) - 1, _iptr(off), int(nboots), int(seed), _dptr(sv),
                                    _dptr(mean), _dptr(cov), _dptr(fcov), _dptr(real))
        self._check(rc, "lqg_bootstrap")
        return dict(mean=mean, fisher_cov=fcov, cov=cov, realizations=real)

    def bootstrap_complete(self, qso_offsets, nboots, seed=0):
        """The complete bootstrap (lqg_bootstrap_complete): mean, cov, the
        realization slots and the number of valid realizations."""
        off = np.ascontiguousarray(qso_offsets, dtype=np.int32)
        nkz = self.nkz
        mean, cov, real = np.zeros(nkz), np.zeros((nkz, nkz)), np.zeros((nboots, nkz))
        nv = C.c_int(0)
        rc = self.lib.lqg_bootstrap_complete(self.h, len(off) - 1, _iptr(off), int(nboots), int(seed), _dptr(mean),
                                             _dptr(cov), _dptr(real), C.byref(nv))
        self._check(rc, "lqg_bootstrap_complete")
        return dict(mean=mean, cov=cov, realizations=real, n_valid=nv.value)

    def clear(self):
        self._check(self.lib.lqg_batch_clear(self.h), "lqg_batch_clear")

    @property
    def size(self):
        return self.lib.lqg_batch_size(self.h)

    def chunk_info(self, i):
        info = np.zeros(8, dtype=np.int32)
        self._check(self.lib.lqg_chunk_info(self.h, i, _iptr(info)), "lqg_chunk_info")
        keys = ("n", "fisher_index_start", "nq", "kbin_upp", "res_index", "zbin_low", "zbin_upp",
                "input_index")
        return dict(zip(keys, (int(x) for x in info)))

    def _theta(self, theta):
        if theta is None:
            return None
        th = np.ascontiguousarray(theta, dtype=np.float64).ravel()
        if len(th) != self.nkz:
            raise ValueError(f"theta must have {self.nkz} values")
        return th

    def iterate(self, theta=None, precision="fp64"):
        th = self._theta(theta)
        rc = self.lib.lqg_nr_iteration(self.h, _dptr(th), PRECISION[precision])
        self._check(rc, "lqg_nr_iteration")

    def iterate_async(self, theta=None, precision="fp64", stream=None):
        """lqg_nr_iteration_async on a cudaStream_t handle (an int, e.g.
        torch.cuda.Stream.cuda_stream) or None; complete with sync()."""
        th = self._theta(theta)
        rc = self.lib.lqg_nr_iteration_async(self.h, _dptr(th), PRECISION[precision],
                                             None if stream is None else C.c_void_p(stream))
        self._check(rc, "lqg_nr_iteration_async")

    def sync(self):
        self._check(self.lib.lqg_sync(self.h), "lqg_sync")

    def autotune(self, max_rel_err=1e-5, max_chunks=48, flags=0):
        """lqg_autotune on the current batch; returns the table (see tuning())."""
        self._check(self.lib.lqg_autotune(self.h, float(max_rel_err), int(max_chunks), int(flags)), "lqg_autotune")
        return self.tuning()

    def tuning(self):
        """The autotuner's table: rows (ld, whitened form, drain interval, Gram K
        per split, CTA-pair products)."""
        n = self.lib.lqg_tuning_get(self.h, None, 0)
        buf = np.zeros(TUNING_FIELDS * max(n, 1), dtype=np.int32)
        self.lib.lqg_tuning_get(self.h, _iptr(buf), n)
        return buf[:TUNING_FIELDS * n].reshape(n, TUNING_FIELDS)

    def set_tuning(self, table):
        t = np.ascontiguousarray(np.asarray(table, dtype=np.int32).reshape(-1, TUNING_FIELDS))
        self._check(self.lib.lqg_tuning_set(self.h, _iptr(t), len(t)), "lqg_tuning_set")

    def download(self):
        d, b, t = (np.zeros(self.nkz) for _ in range(3))
        f = np.zeros((self.nkz, self.nkz))
        st = np.zeros(max(self.size, 1), dtype=np.int32)
        rc = self.lib.lqg_download(self.h, _dptr(d), _dptr(b), _dptr(t), _dptr(f), _iptr(st))
        self._check(rc, "lqg_download")
        return dict(d=d, b=b, t=t, fisher=f, status=st[:self.size])

    def chunk_result(self, i):
        nq = self.chunk_info(i)["nq"]
        d, b, t = (np.zeros(nq) for _ in range(3))
        f = np.zeros((nq, nq))
        rc = self.lib.lqg_chunk_result(self.h, i, _dptr(d), _dptr(b), _dptr(t), _dptr(f))
        self._check(rc, "lqg_chunk_result")
        return d, b, t, f

    def fisher_solve(self, fisher_sum, dbt):
        n = self.nkz
        fs = np.ascontiguousarray(fisher_sum, dtype=np.float64)
        db = np.ascontiguousarray(dbt, dtype=np.float64)
        if fs.shape != (n, n) or db.shape != (3, n):
            raise ValueError(f"fisher_sum must be {n} x {n} and dbt 3 x {n}")
        out = {k: np.zeros((n, n)) for k in ("fisher", "solver", "inverse")}
        w = np.zeros((3, n))
        th = np.zeros(n)
        damped, dof, damp = C.c_int(), C.c_int(), C.c_double()
        rc = self.lib.lqg_fisher_solve(self.h, _dptr(fs), _dptr(db), _dptr(out["fisher"]),
                                       _dptr(out["solver"]), _dptr(out["inverse"]), _dptr(w),
                                       _dptr(th), C.byref(damped), C.byref(dof), C.byref(damp))
        self._check(rc, "lqg_fisher_solve")
        out.update(weighted=w, theta=th, damped=damped.value, dof=dof.value, damp=damp.value)
        return out

    def timings(self):
        """Device ms of the last iteration: build S/C, factorisation, build Q,
        C^-1 Q products, traces, per-chunk reduction, accumulation, total."""
        ms = np.zeros(8)
        self.lib.lqg_last_timings(self.h, _dptr(ms), 8)
        return ms

    def launch_count(self):
        return self.lib.lqg_last_launch_count(self.h)

    def wave_count(self):
        return self.lib.lqg_last_wave_count(self.h)

    def h2d_bytes(self):
        """Bytes the last iteration copied host to device (lqg_last_h2d_bytes)."""
        v = C.c_int64(0)
        self._check(self.lib.lqg_last_h2d_bytes(self.h, C.byref(v)), "lqg_last_h2d_bytes")
        return int(v.value)

    def set_wait_limit(self, seconds):
        """Limit of the tensor-core kernels' waits (0: the default 2 s)."""
        self._check(self.lib.lqg_set_wait_limit(self.h, float(seconds)), "lqg_set_wait_limit")

    def set_fisher_optimization(self, on=True):
        """Banded chunk Fisher matrices, as lyspeq built with FISHER_OPTIMIZATION."""
        self._check(self.lib.lqg_set_fisher_optimization(self.h, 1 if on else 0), "lqg_set_fisher_optimization")


def probe_fp64_rate(device=0):
    """Measured DFMA throughput of the device, TFLOP/s."""
    lib = load_library()
    out = C.c_double(0.0)
    rc = lib.lqg_probe_fp64_rate(int(device), C.byref(out))
    if rc != LQG_OK:
        raise RuntimeError(f"lqg_probe_fp64_rate failed ({rc})")
    return out.value


def chunk_plan(bins, tables, lam, delta, ivar, offsets, r_fwhm, max_forest_length, max_mean_pixel_size=150.0,
               oversampling=0, resomat=None):
    """What an Engine's add_chunks (resomat None) or add_chunks_reso (resomat:
    one row of nelem values per pixel, with oversampling) would make of the
    chunks, without a context or a GPU (lqg_chunk_plan): per chunk its status
    and, when accepted, the chunk_info fields (a dict as Engine.chunk_info
    returns; None if rejected)."""
    lib = load_library()
    lam, delta, ivar, offsets = Engine._pixel_arrays(lam, delta, ivar, offsets)
    n = len(offsets) - 1
    rm = None
    if resomat is not None:
        rm = np.ascontiguousarray(resomat, dtype=np.float64)
        if rm.ndim != 2 or rm.shape[0] != len(lam):
            raise ValueError("resomat must have one row per pixel")
        r_fwhm = np.zeros(n, dtype=np.int32)
    r_fwhm = np.ascontiguousarray(r_fwhm, dtype=np.int32).ravel()
    if len(r_fwhm) != n:
        raise ValueError("one r_fwhm per chunk")
    k_edges = np.ascontiguousarray(bins.k_edges, dtype=np.float64)
    z = np.ascontiguousarray(bins.z_centers, dtype=np.float64)
    r = np.ascontiguousarray([t.r_fwhm for t in tables], dtype=np.int32)
    dv = np.ascontiguousarray([t.dv for t in tables], dtype=np.float64)
    b = LqgBins(bins.nk, bins.nz, _dptr(k_edges), _dptr(z), bins.dz, 1 if bins.triangular else 0)
    t = LqgTables(len(tables), _iptr(r), _dptr(dv), 2, 1.0, 2, None, None)
    o = LqgOpts(float(max_forest_length), float(max_mean_pixel_size), -1, -1, 0, 0, 0, -1, 0, 0.0)
    status = np.zeros(max(n, 1), dtype=np.int32)
    info = np.zeros(8 * max(n, 1), dtype=np.int32)
    rc = lib.lqg_chunk_plan(C.byref(b), C.byref(t), C.byref(o), n, offsets.ctypes.data_as(C.POINTER(C.c_int64)),
                            _dptr(lam), _dptr(delta), _dptr(ivar), _iptr(r_fwhm), int(oversampling),
                            0 if rm is None else rm.shape[1], _dptr(rm), _iptr(status), _iptr(info))
    if rc != LQG_OK:
        raise RuntimeError(f"lqg_chunk_plan failed ({rc})")
    keys = ("n", "fisher_index_start", "nq", "kbin_upp", "res_index", "zbin_low", "zbin_upp", "input_index")
    return status[:n], [dict(zip(keys, (int(x) for x in info[8 * i:8 * i + 8]))) if status[i] == 0 else None
                        for i in range(n)]


def fisher_solve(fisher_sum, dbt):
    """The Newton-Raphson update from the global sums alone (lqg_fisher_solve_n,
    host only): fisher_sum nkz x nkz (upper triangle, unhalved), dbt 3 x nkz.
    Returns the same dictionary as Engine.fisher_solve."""
    lib = load_library()
    fs = np.ascontiguousarray(fisher_sum, dtype=np.float64)
    db = np.ascontiguousarray(dbt, dtype=np.float64)
    n = fs.shape[0]
    if fs.shape != (n, n) or db.shape != (3, n):
        raise ValueError("fisher_sum must be nkz x nkz and dbt 3 x nkz")
    out = {k: np.zeros((n, n)) for k in ("fisher", "solver", "inverse")}
    w = np.zeros((3, n))
    th = np.zeros(n)
    damped, dof, damp = C.c_int(), C.c_int(), C.c_double()
    rc = lib.lqg_fisher_solve_n(n, _dptr(fs), _dptr(db), _dptr(out["fisher"]), _dptr(out["solver"]),
                                _dptr(out["inverse"]), _dptr(w), _dptr(th), C.byref(damped), C.byref(dof),
                                C.byref(damp))
    if rc != 0:
        raise RuntimeError(f"lqg_fisher_solve_n failed with {rc}")
    out.update(weighted=w, theta=th, damped=damped.value, dof=dof.value, damp=damp.value)
    return out


def bootstrap_coefficients(n_qso, nboots, seed=0, per_realization=False):
    """The Poisson coefficients of the bootstraps, p[q, b] (host only)."""
    lib = load_library()
    p = np.zeros((n_qso, nboots), dtype=np.uint8)
    rc = lib.lqg_bootstrap_coefficients(int(n_qso), int(nboots), int(seed), int(bool(per_realization)),
                                        p.ctypes.data_as(C.POINTER(C.c_ubyte)))
    if rc != LQG_OK:
        raise RuntimeError(f"lqg_bootstrap_coefficients failed with {rc}")
    return p


def smooth_ivar(ivar, sigmapix):
    """Smoother::smoothIvar through the library (host only)."""
    lib = load_library()
    iv = np.ascontiguousarray(ivar, dtype=np.float64)
    out = np.empty_like(iv)
    rc = lib.lqg_smooth_ivar(len(iv), _dptr(iv), int(sigmapix), _dptr(out))
    if rc != LQG_OK:
        raise RuntimeError(f"lqg_smooth_ivar failed with {rc}")
    return out


def resomat_smooth(values, sigmapix):
    """Smoother::smooth1D on each diagonal through the library (host only): values[ndiags][n]."""
    lib = load_library()
    v = np.array(values, dtype=np.float64, order="C")
    nd, n = v.shape
    rc = lib.lqg_resomat_smooth(n, nd, _dptr(v), int(sigmapix))
    if rc != LQG_OK:
        raise RuntimeError(f"lqg_resomat_smooth failed with {rc}")
    return v


def resomat_deconvolve(values, m):
    """DiaMatrix::deconvolve through the library (host only): values[ndiags][n]."""
    lib = load_library()
    v = np.array(values, dtype=np.float64, order="C")
    nd, n = v.shape
    rc = lib.lqg_resomat_deconvolve(n, nd, _dptr(v), float(m))
    if rc != LQG_OK:
        raise RuntimeError(f"lqg_resomat_deconvolve failed with {rc}")
    return v


def resomat_oversample(values, osamp, dlambda):
    """Resolution::oversample through the library (host only): rows[n][nelem]."""
    lib = load_library()
    v = np.ascontiguousarray(values, dtype=np.float64)
    nd, n = v.shape
    rows = np.zeros((n, 2 * (nd // 2) * osamp + 1))
    rc = lib.lqg_resomat_oversample(n, nd, _dptr(v), int(osamp), float(dlambda), _dptr(rows))
    if rc != LQG_OK:
        raise RuntimeError(f"lqg_resomat_oversample failed with {rc}")
    return rows


def generate_tables(bins, rd_pairs, nv, v_length, nzp, fid, with_signal=True, device=0):
    """SQ lookup tables for (R, dv) pairs on the GPU (lqg_tables_generate).
    Returns (deriv [n][nk][nv], signal [n][nv][nzp] or None)."""
    lib = load_library()
    k_edges = np.ascontiguousarray(bins.k_edges, dtype=np.float64)
    zc = np.ascontiguousarray(bins.z_centers, dtype=np.float64)
    b = LqgBins(bins.nk, bins.nz, _dptr(k_edges), _dptr(zc), bins.dz, 1 if bins.triangular else 0)
    r = np.ascontiguousarray([p[0] for p in rd_pairs], dtype=np.int32)
    dv = np.ascontiguousarray([p[1] for p in rd_pairs], dtype=np.float64)
    n = len(rd_pairs)
    deriv = np.zeros((n, bins.nk, nv))
    signal = np.zeros((n, nv, nzp)) if with_signal else None
    f = np.ascontiguousarray(fid, dtype=np.float64)
    rc = lib.lqg_tables_generate(C.byref(b), n, _iptr(r), _dptr(dv), int(nv), float(v_length), int(nzp),
                                 _dptr(f), int(bool(with_signal)), _dptr(deriv),
                                 _dptr(signal) if with_signal else None, int(device))
    if rc != LQG_OK:
        raise RuntimeError(f"lqg_tables_generate failed with {rc}")
    return deriv, signal
