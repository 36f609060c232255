"""Seeded synthetic workloads for the per-chunk QMLE path.

No survey data ships with this project, so every workload is generated here
with the shapes, sizes and value distributions of the named configurations:

* ``small``    : 64 chunks, N uniform-int in [100, 500], dv = 30 km/s,
                 lambda_0 ~ U(3600, 5000) A, R ~ U[2000, 5000] (multiple of 100),
                 sigma_pix ~ lognormal(ln 0.2, 0.3); 20 linear k bins of 2e-3 s/km,
                 3 triangular z bins (centres 2.2, 2.4, 2.6, dz = 0.2).
* ``desi``     : 4096 chunks, N log-uniform in [200, 1200], dv = 50 km/s,
                 R ~ U[2000, 5000], 35 k bins (20 linear dk = 5e-4, 15 log to
                 0.1 s/km), 13 triangular z bins centred 1.8 ... 4.2,
                 S/N per pixel ~ lognormal(ln 1, 0.8), continuum marginalisation
                 of amplitude + slope (ContinuumLogLambdaMargOrder 1).
* ``echelle``  : 512 chunks, N uniform-int in [1000, 4000], dv ~ U[2.5, 5]
                 (rounded to 0.1), R ~ U[30000, 50000], 40 k bins (10 x 5e-4
                 linear, 30 log to 0.2 s/km), 6 z bins centred 2.0 ... 3.0,
                 sigma ~ lognormal(ln 0.05, 0.5).
* ``desi_reso``: 16384 chunks, N log-uniform in [150, 1000] on a grid linear
                 in wavelength with dv = 50 km/s at its first pixel, each with an
                 11-diagonal resolution matrix (Gaussian rows whose width varies
                 by +-10 % smoothly along the spectrum, R ~ U[2000, 5000]),
                 deconvolved (m = 1) and oversampled x 3 by the reader; the k/z
                 binning of ``small``; S/N per pixel ~ lognormal(ln 1, 0.8).
                 One signal table (R = 100000, dv = 16.7) serves every chunk.
* ``tiny_reso`` and ``tiny_reso_dia``: 6 such spectra of 110-180 pixels,
                 oversampled x 3 and deconvolved, or used as diagonal matrices
                 on the pixel grid.

The lookup tables follow the definitions lyspeq tabulates
(core/sq_table.cpp:201-323 with core/fiducial_cosmology.cpp:273-331):

    Q_k(v)   = (1/pi) int_{k1}^{k2} W^2(k) cos(k v) dk
    S(z, v)  = (1/pi) int_0^kmax W^2(k) P_fid(k, z) cos(k v) dk
    W(k)     = sinc(k dv / 2) exp(-k^2 R^2 / 2),  R = c / R_fwhm / 2.35482

evaluated here by composite Gauss-Legendre quadrature (the reference uses GSL
QAWO and an FFT; the tables are inputs of the hot path, so both paths read the
same tabulated numbers).  Spectra are Gaussian realisations of P_fid W^2 at the
chunk's median redshift on a uniform velocity grid plus white noise.
"""
from __future__ import annotations

import dataclasses
import math
import os
import struct

import numpy as np

C_KMS = 299792.458
LYA_REST = 1215.67
ONE_SIGMA_2_FWHM = 2.35482004503
PD13_K0, PD13_Z0 = 0.009, 3.0
PD13_DEFAULT = (6.621420e-02, -2.685349e+00, -2.232763e-01, 3.591244e+00,
                -1.768045e-01, 3.598261e+02)   # A, n, alpha, B, beta, lambda


def pd13_power(k, z, p=PD13_DEFAULT):
    """Palanque-Delabrouille et al. 2013 fit with a Lorentzian damping,
    as core/fiducial_cosmology.cpp:273-282."""
    A, n, alpha, B, beta, lam = p
    q0 = np.asarray(k) / PD13_K0 + 1e-15
    x0 = (1.0 + np.asarray(z)) / (1.0 + PD13_Z0)
    return (A * math.pi / PD13_K0 * q0 ** (2.0 + n + alpha * np.log(q0) + beta * np.log(x0))
            * x0 ** B / (1.0 + lam * np.asarray(k) ** 2))


def window2(k, dv, r_kms):
    """W^2(k): pixel top-hat times Gaussian resolution
    (core/fiducial_cosmology.cpp:305-313)."""
    k = np.asarray(k, dtype=np.float64)
    x = k * dv / 2.0
    sinc = np.where(x == 0, 1.0, np.sin(x) / np.where(x == 0, 1.0, x))
    kr = k * r_kms
    return (sinc * np.exp(-kr * kr / 2.0)) ** 2


@dataclasses.dataclass
class Bins:
    """k and z binning as core/global_numbers.cpp:209-251 builds it."""
    k0: float
    nklin: int
    dklin: float
    nklog: int
    dklog: float
    z0: float
    dz: float
    nz: int
    triangular: bool = True
    klast: float = -1.0

    def __post_init__(self):
        edges = [self.k0 + self.dklin * i for i in range(self.nklin + 1)]
        for i in range(1, self.nklog + 1):
            edges.append(edges[self.nklin] * 10.0 ** (i * self.dklog))
        ktemp = (self.k0 + self.dklin * self.nklin) * 10.0 ** (self.nklog * self.dklog)
        if self.klast > ktemp:
            edges.append(self.klast)
        self.k_edges = np.array(edges)
        self.nk = len(edges) - 1
        self.k_centers = (self.k_edges[:-1] + self.k_edges[1:]) / 2.0
        self.z_centers = np.array([self.z0 + self.dz * m for m in range(self.nz)])
        self.z_lower = self.z_centers[0] - self.dz / 2.0
        self.z_upper = self.z_centers[-1] + self.dz / 2.0
        self.nkz = self.nk * self.nz


@dataclasses.dataclass
class Table:
    """One (R, dv) lookup table in lyspeq's in-memory layout:
    deriv[kn][nv] and signal[nv][nz] (z fastest), core/sq_table.cpp:270, :307."""
    r_fwhm: int
    dv: float
    nv: int
    lenv: float
    nzp: int
    z1: float
    lenz: float
    deriv: np.ndarray
    signal: np.ndarray

    @property
    def dv_table(self):
        return self.lenv / (self.nv - 1)

    @property
    def dz_table(self):
        return self.lenz / (self.nzp - 1)


def _gl_panels(a, b, width, order=8):
    """Nodes and weights of composite Gauss-Legendre on [a, b]."""
    if b <= a:
        return np.zeros(0), np.zeros(0)
    npan = max(1, int(math.ceil((b - a) / width)))
    x, w = np.polynomial.legendre.leggauss(order)
    edges = np.linspace(a, b, npan + 1)
    h = np.diff(edges)[:, None]
    mid = (edges[:-1] + edges[1:])[:, None] / 2.0
    return (mid + h / 2.0 * x[None, :]).ravel(), (h / 2.0 * w[None, :]).ravel()


def _cosine_sums(knodes, weights, v):
    """sum_j weights[j, c] cos(k_j v_n) for a uniform v grid, by blocks:
    cos(k(v0+u)) = cos(k v0) cos(k u) - sin(k v0) sin(k u)."""
    nv = len(v)
    dv = v[1] - v[0] if nv > 1 else 0.0
    blk = 128
    u = np.arange(blk) * dv
    cu, su = np.cos(np.outer(u, knodes)), np.sin(np.outer(u, knodes))
    out = np.empty((nv, weights.shape[1]))
    for s in range(0, nv, blk):
        e = min(nv, s + blk)
        a, b = np.cos(knodes * v[s]), np.sin(knodes * v[s])
        out[s:e] = (cu[:e - s] @ (a[:, None] * weights)) - (su[:e - s] @ (b[:, None] * weights))
    return out


def build_table(bins: Bins, r_fwhm: int, dv: float, nv: int, lenv: float, nzp: int,
                fid=PD13_DEFAULT) -> Table:
    r_kms = C_KMS / r_fwhm / ONE_SIGMA_2_FWHM
    v = 0.0 + (lenv / (nv - 1)) * np.arange(nv)
    z1 = bins.z_centers[0] - bins.dz
    lenz = bins.dz * (bins.nz + 1)
    zgrid = z1 + (lenz / (nzp - 1)) * np.arange(nzp)
    panel = 3.0 / max(lenv, 1.0)
    deriv = np.empty((bins.nk, nv))
    for kn in range(bins.nk):
        kk, ww = _gl_panels(bins.k_edges[kn], bins.k_edges[kn + 1], panel)
        deriv[kn] = _cosine_sums(kk, (ww * window2(kk, dv, r_kms) / math.pi)[:, None], v)[:, 0]
    # Signal: a real inverse FFT of W^2 P on a grid twice as fine as the table,
    # normalised by the box length (core/sq_table.cpp:223-228, :296-310 and
    # mathtools/real_field.cpp:87-92).
    rft_m = 2
    nrft = int(2 ** (math.ceil(math.log2(2 * rft_m * nv)) + 1))
    dx = (lenv / (nv - 1)) / rft_m
    length = dx * nrft
    kgrid = np.arange(nrft // 2 + 1) * (2.0 * math.pi / length)
    signal = np.empty((nv, nzp))
    for iz, z in enumerate(zgrid):
        fk = window2(kgrid, dv, r_kms) * pd13_power(kgrid, z, fid)
        fx = np.fft.irfft(fk, n=nrft) * nrft / length
        signal[:, iz] = fx[rft_m * np.arange(nv)]
    return Table(int(r_fwhm), float(dv), nv, float(lenv), nzp, float(z1), float(lenz), deriv, signal)


@dataclasses.dataclass
class Spectrum:
    """One spectrum as a lyspeq binary file holds it (io/qso_file.hpp:20-37)."""
    wave: np.ndarray     # observed wavelength, Angstrom
    delta: np.ndarray
    sigma: np.ndarray    # noise; the reader turns it into ivar = 1/sigma^2
    r_fwhm: int
    dv: float
    z_qso: float = 3.0
    # resolution matrix in lyspeq's DiaMatrix layout: ndiags x n, diagonal d
    # holds offset ndiags/2 - d, the element of column c at [d, c]
    resomat: np.ndarray | None = None


@dataclasses.dataclass
class Workload:
    name: str
    seed: int
    bins: Bins
    tables: list
    spectra: list
    nv: int
    lenv: float
    nzp: int
    max_forest_length: float
    cont_logl_order: int = -1
    cont_l_order: int = -1
    fid: tuple = PD13_DEFAULT
    reso: bool = False          # UseResoMatrix
    oversample: int = -1        # OversampleRmat
    deconv_m: float = 0.0       # ResoMatDeconvolutionM

    def table_index(self):
        return {(t.r_fwhm, round(t.dv, 1)): i for i, t in enumerate(self.tables)}


def _gaussian_field(rng, n, dv, r_kms, z, fid):
    m = 1 << int(math.ceil(math.log2(2 * n)))
    k = 2.0 * math.pi * np.fft.rfftfreq(m, d=dv)
    pk = pd13_power(np.maximum(k, 1e-8), z, fid) * window2(k, dv, r_kms)
    pk[0] = 0.0
    white = np.fft.rfft(rng.standard_normal(m))
    field = np.fft.irfft(white * np.sqrt(pk / dv), n=m)
    return field[:n]


def gaussian_resomat(n: int, sigma_pix: np.ndarray, ndiags: int = 11) -> np.ndarray:
    """Resolution matrix with Gaussian rows of width sigma_pix[i] (pixels),
    each row normalised to unit sum over its ndiags entries, in lyspeq's
    DiaMatrix layout (mathtools/matrix_helper.cpp:503-520): values[d, c] is
    the element of row c - off(d), column c, off(d) = ndiags/2 - d; entries
    whose row falls outside the spectrum are zero."""
    noff = ndiags // 2
    offs = np.arange(noff, -noff - 1, -1)
    rows = np.exp(-0.5 * (offs[None, :] / sigma_pix[:, None]) ** 2)   # [row i, d]
    rows /= rows.sum(axis=1, keepdims=True)
    vals = np.zeros((ndiags, n))
    for d, off in enumerate(offs):
        r = np.arange(n) - off          # row of column c on this diagonal
        ok = (r >= 0) & (r < n)
        vals[d, ok] = rows[r[ok], d]
    return vals


def _make_reso_workload(name, rng, seed, nch):
    """The resolution-matrix workloads (see the module docstring)."""
    bins = Bins(0.0, 20, 2e-3, 0, 0.0, 2.2, 0.2, 3)
    dv = 50.0
    if name == "desi_reso":
        npix = np.exp(rng.uniform(math.log(150), math.log(1000), size=nch)).astype(int)
    else:
        npix = rng.integers(110, 181, size=nch)
    span = 1.0 + npix * dv / C_KMS
    lmin, lmax = LYA_REST * (1 + bins.z_lower) * 1.0005, LYA_REST * (1 + bins.z_upper) * 0.9995
    lam0 = rng.uniform(lmin, lmax / span)
    rs = (np.round(rng.uniform(2000, 5000, size=nch) / 100) * 100).astype(int)
    spectra = []
    for i in range(nch):
        n = int(npix[i])
        dlam = lam0[i] * dv / C_KMS
        wave = lam0[i] + dlam * np.arange(n)
        zmed = float(np.median(wave)) / LYA_REST - 1.0
        r_kms = C_KMS / rs[i] / ONE_SIGMA_2_FWHM
        sig = 1.0 / np.exp(rng.normal(0.0, 0.8, size=n))
        delta = _gaussian_field(rng, n, dv, r_kms, zmed, PD13_DEFAULT) + sig * rng.standard_normal(n)
        sigma_pix = wave / rs[i] / ONE_SIGMA_2_FWHM / dlam
        phase = rng.uniform(0.0, 2.0 * math.pi)
        sigma_pix = sigma_pix * (1.0 + 0.1 * np.sin(2.0 * math.pi * np.arange(n) / n + phase))
        spectra.append(Spectrum(wave, delta, sig, int(rs[i]), dv, resomat=gaussian_resomat(n, sigma_pix)))
    osamp = -1 if name == "tiny_reso_dia" else 3
    table_dv = round(dv / 3.0, 1)
    longest = max(float(np.log(s.wave[-1] / s.wave[0]) * C_KMS) for s in spectra)
    # MaximumForestLength such that no chunk is too short (150 pixels of 50 km/s
    # at 0.45 of it), as the other workloads choose it
    mfl = 15000.0 if name == "desi_reso" else 6000.0
    lenv = float(math.ceil(max(longest + 12 * dv, mfl) * 1.02 / 100.0) * 100.0)
    nv = int(math.ceil(lenv / (table_dv / 2.0))) + 1
    nzp = max(10, bins.nz + 2)
    tables = [build_table(bins, 100000, table_dv, nv, lenv, nzp)]
    return Workload(name, seed, bins, tables, spectra, nv, lenv, nzp, mfl, -1, -1,
                    reso=True, oversample=osamp, deconv_m=1.0)


def make_workload(name: str, seed: int | None = None, n_chunks: int | None = None) -> Workload:
    """Build one of the named synthetic workloads."""
    seeds = {"small": 20240601, "desi": 20240602, "echelle": 20240604, "tiny": 20240605,
             "desi_reso": 20240606, "tiny_reso": 20240607, "tiny_reso_dia": 20240607,
             "echelle_small": 20240608}
    seed = seeds[name] if seed is None else seed
    rng = np.random.Generator(np.random.PCG64(seed))
    if name in ("desi_reso", "tiny_reso", "tiny_reso_dia"):
        nch = (16384 if name == "desi_reso" else 6) if n_chunks is None else n_chunks
        return _make_reso_workload(name, rng, seed, nch)
    if name in ("small", "tiny"):
        bins = Bins(0.0, 20, 2e-3, 0, 0.0, 2.2, 0.2, 3)
        nch = 64 if name == "small" else 6
        nch = nch if n_chunks is None else n_chunks
        lo, hi = (100, 500) if name == "small" else (100, 180)
        dv = 30.0
        npix = rng.integers(lo, hi + 1, size=nch)
        # lambda_0 ~ U(3600, 5000) as specified; the tiny case keeps chunks inside the z range
        lam0 = rng.uniform(3600.0, 5000.0, size=nch) if name == "small" else \
            rng.uniform(LYA_REST * 3.12, LYA_REST * 3.55, size=nch)
        rs = (np.round(rng.uniform(2000, 5000, size=nch) / 100) * 100).astype(int)
        sig = [np.exp(rng.normal(math.log(0.2), 0.3, size=n)) for n in npix]
        dvs = np.full(nch, dv)
        mfl = 6000.0
        cont = (-1, -1)
    elif name == "desi":
        bins = Bins(0.0, 20, 5e-4, 15, 1.0 / 15.0, 1.8, 0.2, 13)
        nch = 4096 if n_chunks is None else n_chunks
        dv = 50.0
        npix = np.exp(rng.uniform(math.log(200), math.log(1200), size=nch)).astype(int)
        span = np.exp(npix * dv / C_KMS)
        lmin, lmax = LYA_REST * (1 + bins.z_lower) * 1.0005, LYA_REST * (1 + bins.z_upper) * 0.9995
        lam0 = rng.uniform(lmin, lmax / span)
        rs = (np.round(rng.uniform(2000, 5000, size=nch) / 100) * 100).astype(int)
        sig = [1.0 / np.exp(rng.normal(0.0, 0.8, size=n)) for n in npix]
        dvs = np.full(nch, dv)
        mfl = 20000.0
        cont = (1, -1)
    elif name in ("echelle", "echelle_small"):
        # echelle_small: the echelle-like set's binning, resolution and noise
        # with N uniform-int in [1000, 1500] (the reference runs it in seconds)
        dklog = math.log10(0.2 / 0.005) / 30.0
        bins = Bins(0.0, 10, 5e-4, 30, dklog, 2.0, 0.2, 6)
        nch = (512 if name == "echelle" else 3) if n_chunks is None else n_chunks
        npix = rng.integers(1000, 4001, size=nch) if name == "echelle" else rng.integers(1000, 1501, size=nch)
        dvs = np.round(rng.uniform(2.5, 5.0, size=nch), 1)
        span = np.exp(npix * dvs / C_KMS)
        lmin, lmax = LYA_REST * (1 + bins.z_lower) * 1.0005, LYA_REST * (1 + bins.z_upper) * 0.9995
        lam0 = rng.uniform(lmin, lmax / span)
        rs = (np.round(rng.uniform(30000, 50000, size=nch) / 100) * 100).astype(int)
        sig = [np.exp(rng.normal(math.log(0.05), 0.5, size=n)) for n in npix]
        mfl = 4000.0
        cont = (-1, -1)
    else:
        raise ValueError(f"unknown workload {name!r}")

    spectra = []
    for i in range(nch):
        n, d = int(npix[i]), float(dvs[i])
        wave = lam0[i] * np.exp(np.arange(n) * d / C_KMS)
        zmed = float(np.median(wave)) / LYA_REST - 1.0
        r_kms = C_KMS / rs[i] / ONE_SIGMA_2_FWHM
        delta = _gaussian_field(rng, n, d, r_kms, zmed, PD13_DEFAULT)
        delta = delta + sig[i] * rng.standard_normal(n)
        spectra.append(Spectrum(wave, delta, sig[i], int(rs[i]), d))

    longest = max(float(np.log(s.wave[-1] / s.wave[0]) * C_KMS) for s in spectra)
    lenv = float(math.ceil(max(longest, mfl) * 1.02 / 100.0) * 100.0)
    min_dv = float(min(dvs))
    nv = int(math.ceil(lenv / (min_dv / 2.0))) + 1
    nzp = max(10, bins.nz + 2)
    pairs = sorted({(int(s.r_fwhm), round(float(s.dv), 1)) for s in spectra})
    tables = [build_table(bins, r, d, nv, lenv, nzp) for r, d in pairs]
    return Workload(name, seed, bins, tables, spectra, nv, lenv, nzp, mfl, cont[0], cont[1])


# ----------------------------------------------------------------------------
# Writers for lyspeq's own file formats (used to run the reference on the same
# inputs).

_DAT_HEADER = struct.Struct("<i4xdddi4xdddddd")   # 88 bytes, io/qso_file.hpp:20-37


def write_dat(path: str, s: Spectrum):
    n = len(s.wave)
    hdr = _DAT_HEADER.pack(n, s.z_qso, 0.0, 0.0, int(s.r_fwhm), 1.0, float(s.dv),
                           float(s.wave[0]), float(s.wave[-1]),
                           float(s.wave[0]) / (1 + s.z_qso), float(s.wave[-1]) / (1 + s.z_qso))
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(np.ascontiguousarray(s.wave, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(s.delta, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(s.sigma, dtype="<f8").tobytes())


def write_resomat(path: str, values: np.ndarray):
    """Side file of a binary spectrum holding its resolution matrix for the
    oracle driver: int32 n, int32 ndiags, then values[ndiags][n] as doubles."""
    nd, n = values.shape
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", n, nd))
        f.write(np.ascontiguousarray(values, dtype="<f8").tobytes())


def read_dat(path: str) -> Spectrum:
    with open(path, "rb") as f:
        buf = f.read()
    n, z, _dec, _ra, r, _snr, dv = _DAT_HEADER.unpack_from(buf, 0)[:7]
    a = np.frombuffer(buf, dtype="<f8", count=3 * n, offset=_DAT_HEADER.size)
    return Spectrum(a[:n].copy(), a[n:2 * n].copy(), a[2 * n:].copy(), r, dv, z)


def _fits_card(key, value=None, string=False):
    if value is None:
        return key.ljust(80)
    if string:
        v = ("'" + str(value).ljust(8) + "'").ljust(20)
    elif isinstance(value, bool):
        v = ("T" if value else "F").rjust(20)
    elif isinstance(value, (int, np.integer)):
        v = str(int(value)).rjust(20)
    else:
        v = repr(float(value)).upper().rjust(20)
    return (key.ljust(8) + "= " + v).ljust(80)


def _fits_hdu(cards, data=None):
    hdr = "".join(cards) + "END".ljust(80)
    hdr += " " * (-len(hdr) % 2880)
    raw = b"" if data is None else np.ascontiguousarray(data, dtype=">f8").tobytes()
    return hdr.encode("ascii") + raw + b"\0" * (-len(raw) % 2880)


def write_table_fits(path: str, t: Table, bins: Bins):
    """SQ table in lyspeq's FITS layout (io/sq_lookup_table_file.cpp:68-155):
    primary HDU METADATA with the header keys, DERIVATIVE and SIGNAL image
    HDUs whose raw buffers are deriv[kn][nv] and signal[nv][nz]."""
    prim = [_fits_card("SIMPLE", True), _fits_card("BITPIX", -64), _fits_card("NAXIS", 1),
            _fits_card("NAXIS1", 0), _fits_card("EXTEND", True),
            _fits_card("EXTNAME", "METADATA", True), _fits_card("NVPTS", t.nv),
            _fits_card("NZPTS", t.nzp), _fits_card("LENV", t.lenv), _fits_card("Z1", t.z1),
            _fits_card("LENZ", t.lenz), _fits_card("RFWHM", t.r_fwhm), _fits_card("DV", t.dv),
            _fits_card("K1", bins.k0), _fits_card("DKLIN", bins.dklin),
            _fits_card("DKLOG", bins.dklog), _fits_card("NKLIN", bins.nklin),
            _fits_card("NKLOG", bins.nklog)]
    out = _fits_hdu(prim)
    for ext, ax, arr in (("DERIVATIVE", (bins.nk, t.nv), t.deriv), ("SIGNAL", (t.nzp, t.nv), t.signal)):
        cards = [_fits_card("XTENSION", "IMAGE", True), _fits_card("BITPIX", -64),
                 _fits_card("NAXIS", 2), _fits_card("NAXIS1", ax[0]), _fits_card("NAXIS2", ax[1]),
                 _fits_card("PCOUNT", 0), _fits_card("GCOUNT", 1), _fits_card("EXTNAME", ext, True)]
        out += _fits_hdu(cards, arr.ravel())
    with open(path, "wb") as f:
        f.write(out)


def read_table_fits(path: str, nk: int | None = None) -> dict:
    """Read a lyspeq SQ table FITS file (any writer) into arrays."""
    with open(path, "rb") as f:
        buf = f.read()
    pos, hdus = 0, []
    while pos + 2880 <= len(buf):
        cards, end = {}, False
        while not end:
            c = buf[pos:pos + 80].decode("ascii")
            pos += 80
            key = c[:8].strip()
            if key == "END":
                end = True
            elif c[8:10] == "= ":
                val = c[10:].split("/")[0].strip() if "'" not in c[10:] else c[10:].split("'")[1].strip()
                cards[key] = val
        pos += -pos % 2880
        naxis = int(cards.get("NAXIS", 0))
        nel = int(np.prod([int(cards[f"NAXIS{i}"]) for i in range(1, naxis + 1)])) if naxis else 0
        nbytes = abs(int(cards.get("BITPIX", 8))) // 8 * nel
        data = np.frombuffer(buf, dtype=">f8", count=nbytes // 8, offset=pos).astype(np.float64)
        pos += nbytes + (-nbytes % 2880)
        hdus.append((cards, data))
    meta = next(c for c, _ in hdus if c.get("EXTNAME") == "METADATA")
    deriv = next(d for c, d in hdus if c.get("EXTNAME") == "DERIVATIVE")
    signal = next(d for c, d in hdus if c.get("EXTNAME") == "SIGNAL")
    nv, nzp = int(meta["NVPTS"]), int(meta["NZPTS"])
    return dict(nv=nv, nzp=nzp, lenv=float(meta["LENV"]), z1=float(meta["Z1"]),
                lenz=float(meta["LENZ"]), r_fwhm=int(meta["RFWHM"]), dv=float(meta["DV"]),
                deriv=deriv.reshape(-1, nv), signal=signal.reshape(nv, nzp))


def write_reference_inputs(w: Workload, outdir: str, marg=None) -> str:
    """Write spectra, tables, lists and a config that lyspeq's LyaPowerEstimate
    reads; returns the config path."""
    os.makedirs(outdir, exist_ok=True)
    spec_dir = os.path.join(outdir, "spectra")
    os.makedirs(spec_dir, exist_ok=True)
    names = []
    for i, s in enumerate(w.spectra):
        nm = f"chunk{i:05d}.dat"
        write_dat(os.path.join(spec_dir, nm), s)
        if w.reso:
            write_resomat(os.path.join(spec_dir, nm + ".rmat"), s.resomat)
        names.append(nm)
    with open(os.path.join(outdir, "flist.txt"), "w") as f:
        f.write(f"{len(names)}\n" + "\n".join(names) + "\n")
    with open(os.path.join(outdir, "slist.txt"), "w") as f:
        f.write(f"{len(w.tables)}\n" + "".join(f"{t.r_fwhm} {t.dv:.1f}\n" for t in w.tables))
    for t in w.tables:
        write_table_fits(os.path.join(outdir, f"signal_R{t.r_fwhm}_dv{t.dv:.1f}.fits"), t, w.bins)
    b = w.bins
    logl, lam = (w.cont_logl_order, w.cont_l_order) if marg is None else marg
    fid = w.fid
    cfg = f"""K0 {b.k0!r}
NumberOfLinearBins {b.nklin}
NumberOfLog10Bins {b.nklog}
LinearKBinWidth {b.dklin!r}
Log10KBinWidth {b.dklog!r}
FirstRedshiftBinCenter {b.z0!r}
RedshiftBinWidth {b.dz!r}
NumberOfRedshiftBins {b.nz}
RedshiftBinningMethod {1 if b.triangular else 0}
FileNameList {outdir}/flist.txt
FileInputDir {spec_dir}/
MaximumForestLength {w.max_forest_length!r}
DynamicChunkNumber 1
OutputDir {outdir}/
LookUpTableDir {outdir}/
OutputFileBase qmle
FileNameRList {outdir}/slist.txt
NumberVPoints {w.nv}
NumberZPoints {w.nzp}
VelocityLength {w.lenv!r}
TurnOffBaseline -1
SmoothLnkLnP 0
FiducialAmplitude {fid[0]!r}
FiducialSlope {fid[1]!r}
FiducialCurvature {fid[2]!r}
FiducialRedshiftPower {fid[3]!r}
FiducialRedshiftCurvature {fid[4]!r}
FiducialLorentzianLambda {fid[5]!r}
InputIsDeltaFlux 1
ContinuumLogLambdaMargOrder {logl}
ContinuumLambdaMargOrder {lam}
NumberOfIterations 1
NumberOfBoots 0
SmoothNoiseWeights -1
AllocatedMemoryMB 200000.
TemporaryFolder {outdir}
OversampleRmat {w.oversample}
ResoMatDeconvolutionM {w.deconv_m!r}
"""
    path = os.path.join(outdir, "qmle.config")
    with open(path, "w") as f:
        f.write(cfg)
    return path
