"""Loader of the golden fixtures written by tests/golden/make_golden.py."""
from __future__ import annotations

import dataclasses
import os

import numpy as np

from lyspeq_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["tiny_nomarg", "tiny_marg1", "tiny_marg3", "tiny_masked", "small_cfg", "desi_sub",
         "tiny_reso", "tiny_reso_dia", "tiny_smooth", "tiny_smooth_mean", "tiny_reso_growth",
         "tiny_reso_smooth", "tiny_tophat", "tiny_nosfid"]
RESO_CASES = ["tiny_reso", "tiny_reso_dia", "tiny_reso_growth", "tiny_reso_smooth"]
# from the reference built with FISHER_OPTIMIZATION (banded chunk Fisher
# matrices); kept out of CASES, whose tests run the full matrices
FOPT_CASES = ["desi_fopt"]
# DESI-size chunks with resolution matrices; kept out of CASES and RESO_CASES
# (their GPU check is tests/test_zzz_reso_sizes.py)
RESO_SIZE_CASES = ["desi_reso_sub"]


@dataclasses.dataclass
class GoldenCase:
    name: str
    bins: synth.Bins
    tables: list
    nv: int
    lenv: float
    nzp: int
    max_forest_length: float
    marg: tuple
    chunks: list          # (lambda_angstrom, delta, ivar, r_fwhm)
    meta: list            # (n, fisher_index_start, nq, kbin_upp, r_fwhm, status)
    dbt: list             # per chunk 3 x nq
    fisher: list          # per chunk nq x nq
    g: dict               # global reference results
    complete: bool
    # resolution-matrix cases: (oversampling, deconvolution m), per chunk the
    # matrix as the reference's chunk holds it and (spectrum, first pixel),
    # per spectrum (lambda, raw DiaMatrix values)
    boot: dict | None = None   # FastBootstrap: mean, cov, realizations, qso of each chunk, n_qso
    nr: dict | None = None     # full NR loop: iterations and the estimator's final state
    reso: tuple | None = None
    rmats: list | None = None
    src: list | None = None
    spectra: list | None = None
    # SmoothNoiseWeights, RedshiftGrowthOn and its exponent, TurnOffBaseline, as Engine keywords
    opts: dict = dataclasses.field(default_factory=lambda: dict(smooth_noise_weights=-1, redshift_growth=False,
                                                                  fid_b=0.0, turn_off_sfid=False))
    smooth_rmat: bool = False
    fisher_optimization: bool = False   # the reference was built with FISHER_OPTIMIZATION

    def port_settings(self, P):
        """The oracle's Settings for this case."""
        return P.Settings(max_forest_length=self.max_forest_length, cont_logl_order=self.marg[0],
                          cont_l_order=self.marg[1], smooth_noise_weights=self.opts["smooth_noise_weights"],
                          redshift_growth=self.opts["redshift_growth"], growth_b=self.opts["fid_b"],
                          turn_off_sfid=self.opts["turn_off_sfid"],
                          fisher_optimization=self.fisher_optimization)


_cache = {}


def load(name: str) -> GoldenCase:
    if name in _cache:
        return _cache[name]
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    b = z["bins"]
    bins = synth.Bins(b[0], int(b[1]), b[2], int(b[3]), b[4], b[5], b[6], int(b[7]), bool(b[8]))
    nv, lenv, nzp, mfl, m0, m1 = z["grid"]
    nv, nzp = int(nv), int(nzp)
    tables = [synth.build_table(bins, int(r), float(dv), nv, float(lenv), nzp)
              for r, dv in zip(z["table_r"], z["table_dv"])]
    sums = np.array([[np.abs(t.deriv).sum(), np.abs(t.signal).sum()] for t in tables])
    np.testing.assert_allclose(sums, z["table_sums"], rtol=1e-12)
    n = int(z["n_chunks"])
    chunks, meta, dbt, fis = [], [], [], []
    for i in range(n):
        m = z[f"c{i}_meta"]
        chunks.append((z[f"c{i}_lam"], z[f"c{i}_delta"], z[f"c{i}_ivar"], int(m[4])))
        meta.append(tuple(int(x) for x in m))
        dbt.append(z[f"c{i}_dbt"])
        fis.append(z[f"c{i}_fisher"])
    g = {k[2:]: z[k] for k in z.files if k.startswith("g_")}
    case = GoldenCase(name, bins, tables, nv, float(lenv), nzp, float(mfl), (int(m0), int(m1)),
                      chunks, meta, dbt, fis, g, bool(z["g_complete"]))
    if "opts" in z.files:
        o = z["opts"]
        case.opts = dict(smooth_noise_weights=int(o[0]), redshift_growth=bool(o[1] > 0), fid_b=float(o[2]),
                         turn_off_sfid=bool(len(o) > 4 and o[4] > 0))
        # SmoothResolutionMatrix: applied while the matrices are prepared
        case.smooth_rmat = len(o) > 3 and o[3] > 0 and o[0] >= 0
    case.fisher_optimization = "fisher_opt" in z.files and bool(z["fisher_opt"])
    if "it_n" in z.files:
        case.nr = dict(n=int(z["it_n"]), theta=z["it_theta"], previous=z["it_prev"], fits=z["it_fits"],
                       fisher=z["it_fisher"], inverse=z["it_inverse"], dbt=z["it_dbt"])
    if "boot_mean" in z.files:
        case.boot = dict(mean=z["boot_mean"], cov=z["boot_cov"], real=z["boot_real"],
                         qso=z["boot_qso"], n_qso=int(z["boot_nqso"]),
                         complete=bool(z["boot_complete"][0]) if "boot_complete" in z.files else False,
                         valid=int(z["boot_complete"][1]) if "boot_complete" in z.files else len(z["boot_real"]))
    if "reso" in z.files:
        case.reso = (int(z["reso"][0]), float(z["reso"][1]))
        case.rmats = [z[f"c{i}_rmat"] for i in range(n)]
        case.src = [tuple(int(x) for x in z[f"c{i}_src"]) for i in range(n)]
        case.spectra = [(z[f"s{j}_lam"], z[f"s{j}_resomat"]) for j in range(int(z["n_spectra"]))]
    _cache[name] = case
    return case


def rel_err(x, ref):
    """max |x - ref| / max |ref|, the error measure of the parity tests."""
    x, ref = np.asarray(x), np.asarray(ref)
    scale = np.max(np.abs(ref))
    if scale == 0:
        return float(np.max(np.abs(x)))
    return float(np.max(np.abs(x - ref)) / scale)


def fisher_err(f, ref):
    """Per-element error of a Fisher matrix normalised by sqrt(F_ii F_jj)."""
    d = np.sqrt(np.abs(np.diag(ref)))
    den = np.outer(d, d)
    den[den == 0] = 1.0
    return float(np.max(np.abs(np.asarray(f) - ref) / den))


def elem_err(x, ref, floor=1e-3):
    """Largest per-element relative error |x_k - ref_k| / |ref_k| over the
    elements with |ref_k| above floor * max |ref| (the others are zero or at a
    zero crossing, where a relative error says nothing)."""
    x, ref = np.asarray(x), np.asarray(ref)
    m = np.abs(ref) > floor * np.max(np.abs(ref))
    if not m.any():
        return 0.0
    return float(np.max(np.abs(x - ref)[m] / np.abs(ref)[m]))


def p1d_err(bins, g_ref, g_mix, fsum, nsig=5.0):
    """Per-bin relative error of P1D = P_fid(k_c, z_c) + theta against the
    reference solution, over the bins measured at nsig sigma or more
    (sigma = sqrt(diag F^-1)); (error, number of such bins).  On the other
    bins the estimate is noise and its relative error says nothing."""
    pfid = synth.pd13_power(np.tile(bins.k_centers, bins.nz), np.repeat(bins.z_centers, bins.nk))
    p_ref, p_mix = pfid + np.asarray(g_ref["theta"]), pfid + np.asarray(g_mix["theta"])
    sig = np.sqrt(np.abs(np.diag(g_ref["inverse"])))
    good = (np.diag(fsum) > 0) & (sig > 0) & (np.abs(p_ref) > nsig * sig)
    if not good.any():
        return 0.0, 0
    return float(np.max(np.abs(p_mix - p_ref)[good] / np.abs(p_ref)[good])), int(good.sum())


def global_sums(case):
    """Global Fisher sum (upper, unhalved) and d, b, t of a fixture's chunks,
    accumulated as Chunk::oneQSOiteration does (core/chunk_estimate.cpp:893-903)."""
    nkz = case.bins.nkz
    fsum, dbt = np.zeros((nkz, nkz)), np.zeros((3, nkz))
    for m, x, f in zip(case.meta, case.dbt, case.fisher):
        fis, nq = m[1], m[2]
        fsum[fis:fis + nq, fis:fis + nq] += f
        dbt[:, fis:fis + nq] += x
    return fsum, dbt
