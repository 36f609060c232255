"""CPU restatement of lyspeq's per-chunk QMLE path (test infrastructure).

This module is the oracle that travels: it re-states, in numpy with the same
LAPACK/BLAS routines (through scipy's bundled OpenBLAS), what lyspeq's C++
does for one Newton-Raphson iteration.  It is imported only by the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``, always as
the checker or the reported CPU baseline, never as the product path.

Parity of this restatement is pinned against the reference itself, compiled
from its own sources (oracle/refbuild), on identical inputs; the reference
build is in turn pinned against lyspeq's golden files
(tests/truth/test_it1_*.dat).

Each step cites the reference lines it follows.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np
from scipy import sparse
from scipy.linalg import lapack

C_KMS = 299792.458
LYA_REST = 1215.67
DOUBLE_EPSILON = 1e-15
MIN_PIXELS_IN_FILE = 100          # core/one_qso_estimate.cpp:14


@dataclasses.dataclass
class Settings:
    """The config values the per-chunk path reads (core/global_numbers.cpp:93-173)."""
    max_forest_length: float = 3.5e4
    number_of_chunks: int = 1
    max_pixel_length_v: float = 150.0
    cont_logl_order: int = 1
    cont_l_order: int = -1
    turn_off_sfid: bool = False
    smooth_noise_weights: int = -1   # SmoothNoiseWeights (mathtools/smoother.hpp:8-9)
    redshift_growth: bool = False    # RedshiftGrowthOn > 0 (core/global_numbers.cpp:127)
    growth_b: float = 0.0            # FIDUCIAL_PD13_PARAMS.B
    fisher_optimization: bool = False   # built with -DFISHER_OPTIMIZATION (configure --enable-fisher-optimization)
    # flux -> delta_F of the input (conv::readConversion, core/fiducial_cosmology.cpp:33-83)
    input_is_delta_flux: bool = True    # InputIsDeltaFlux > 0
    use_chunks_mean_flux: bool = False  # UseChunksMeanFlux > 0
    mean_flux: tuple | None = None      # (z, F-bar) of a MeanFluxFile

    @property
    def max_forest_length_v(self):
        return self.max_forest_length / max(1, self.number_of_chunks)

    @property
    def min_forest_length_v(self):
        return 0.90 / 2 * self.max_forest_length_v

    @property
    def cont_nvecs(self):
        # core/global_numbers.cpp:78-90
        if self.cont_logl_order >= 0 or self.cont_l_order >= 0:
            n = 1
            if self.cont_logl_order > 0:
                n += self.cont_logl_order
            if self.cont_l_order > 0:
                n += self.cont_l_order
            return n
        return 0


@dataclasses.dataclass
class ChunkData:
    """Host-side chunk, as Chunk::Chunk leaves it (core/chunk_estimate.cpp:141-257)."""
    wave: np.ndarray           # lambda / LYA_REST
    delta: np.ndarray
    ivar: np.ndarray
    r_fwhm: int
    dv: float
    res_index: int
    kbin_upp: int
    zbin_low: int
    zbin_upp: int
    nq: int
    fisher_index_start: int
    # resolution matrix (UseResoMatrix): dense R (n x ncols) and the grid the
    # signal and derivative matrices are evaluated on before R . M . R^T
    # (lambda / LYA_REST, ncols points); None without a resolution matrix
    rmat: np.ndarray | None = None
    fine_wave: np.ndarray | None = None

    @property
    def n(self):
        return len(self.wave)


def _median_sorted(a):
    n = len(a)
    return (a[n // 2 - 1] + a[n // 2]) / 2 if n % 2 == 0 else a[n // 2]


def _median(v):
    return _median_sorted(np.sort(v))


def _c_round(x):
    return math.floor(x + 0.5) if x >= 0 else math.ceil(x - 0.5)


def find_redshift_bin(bins, z):
    """core/global_numbers.cpp:344-355."""
    if z < bins.z_lower:
        return -1
    r = int((z - bins.z_lower) / bins.dz)
    return min(r, bins.nz)


def cut_masked_boundary(ivar):
    """QSOFile::_cutMaskedBoundary, io/qso_file.cpp:139-157: (start, stop)."""
    nz = np.flatnonzero(ivar != 0)
    if len(nz) == 0:
        raise ValueError("Empty spectrum when masked pixels at boundary are removed!")
    return int(nz[0]), int(nz[-1]) + 1


def preprocess_spectrum(spec, bins, reso=None, settings=None):
    """Reading and cleaning of one binary spectrum: io/qso_file.cpp:352-369
    (sigma -> ivar), :189-230 (maskOutliers), :159-187 (cutBoundary) and
    core/one_qso_estimate.cpp:52-100.  Returns (wave, delta, ivar) in
    Angstrom, or raises ValueError when the reference would drop the file.
    With reso = (oversampling, deconvolution m[, smoothing sigma]) the
    spectrum's resolution matrix is smoothed (sigma >= 0:
    SmoothResolutionMatrix with SmoothNoiseWeights sigma), deconvolved and
    oversampled before the cut (core/one_qso_estimate.cpp:75-89) and a fourth
    item, the matrix cut with the pixels (rows [n][nelem] when oversampled,
    else values[ndiags][n]), is returned."""
    wave = np.array(spec.wave, dtype=np.float64)
    delta = np.array(spec.delta, dtype=np.float64)
    ivar = 1.0 / (np.asarray(spec.sigma, dtype=np.float64) ** 2)
    ivar[ivar < DOUBLE_EPSILON] = 0.0
    # flux -> delta_F (core/one_qso_estimate.cpp:62-65)
    convert_flux_to_delta(settings, wave, delta, ivar)
    # maskOutliers (factor 5)
    good = ivar != 0
    realsize = int(good.sum())
    tmp = delta[good]
    med = _median(tmp.copy())
    mad = 1.4826 * (1.0 + 1.0 / math.sqrt(realsize)) * _median(np.abs(tmp - med))
    mad = max(1.0, mad)
    for i in np.flatnonzero(good):
        s = 5.0 * max(1.0 / math.sqrt(ivar[i]), mad)
        fup = math.exp(1.663e-03 * (wave[i] / LYA_REST) ** 4.107)
        if delta[i] < (-1.0 - s) or delta[i] > (fup + s):
            delta[i] = 0.0
            ivar[i] = 0.0
    rm = None
    if reso is not None:
        osamp, m = reso[:2]
        vals = np.array(spec.resomat, dtype=np.float64)
        if len(reso) > 2 and reso[2] >= 0:
            vals = smooth_rows(vals, reso[2])
        if m > 0:
            vals = dia_deconvolve(vals, m)
        if osamp > 0:
            dlam = _median(np.diff(wave))          # QSOFile::readData, io/qso_file.cpp:124-128
            rm = dia_oversample(vals, osamp, dlam)
        else:
            rm = vals
    # cutBoundary
    l1, l2 = LYA_REST * (1 + bins.z_lower), LYA_REST * (1 + bins.z_upper)
    wi1 = int(np.searchsorted(wave, l1, side="left"))
    wi2 = int(np.searchsorted(wave, l2, side="right"))
    if wi1 == len(wave) or wi2 == 0:
        raise ValueError("Empty spectrum when redshift boundary is applied!")
    wave, delta, ivar = wave[wi1:wi2], delta[wi1:wi2], ivar[wi1:wi2]
    a, b = cut_masked_boundary(ivar)
    wave, delta, ivar = wave[a:b], delta[a:b], ivar[a:b]
    if int((ivar != 0).sum()) < MIN_PIXELS_IN_FILE:
        raise ValueError("Short file")
    if reso is None:
        return wave, delta, ivar
    lo, hi = wi1 + a, wi1 + b
    rm = rm[lo:hi] if reso[0] > 0 else rm[:, lo:hi]
    return wave, delta, ivar, rm


# ---------------------------------------------------------------------------
# Resolution matrices (mathtools/matrix_helper.cpp:503-1095, real_field.cpp:78-110)

def dia_row_indices(i, n, ndiags):
    """DiaMatrix::_getRowIndices, mathtools/matrix_helper.cpp:608-620: flat
    indices into values[ndiags][n] of row i's entries, columns i - noff ..
    i + noff; entries beyond an edge repeat the mirrored entry of the row."""
    noff = ndiags // 2
    idx = [j * n + (noff - j) + i for j in range(ndiags - 1, -1, -1)]
    if i < noff:
        for j in range(noff - i):
            idx[j] = idx[ndiags - 1 - j]
    elif i > n - noff - 1:
        for j in range(i - n + noff + 1):
            idx[ndiags - 1 - j] = idx[j]
    return idx


def dia_deconvolve(values, m):
    """DiaMatrix::deconvolve (mathtools/matrix_helper.cpp:653-682) with
    RealField::deconvolveSinc (real_field.cpp:78-110): each row, zero-padded by
    5 on both sides, is divided by sinc(pi m i / size) in Fourier space."""
    nd, n = values.shape
    flat = values.ravel()
    pad = 5
    size = nd + 2 * pad
    for i in range(n):
        idx = dia_row_indices(i, n, nd)
        x = np.zeros(size)
        x[pad:pad + nd] = flat[idx]
        fk = np.fft.rfft(x)
        for k in range(1, size // 2 + 1):
            a = math.pi * m * k / size
            fk[k] /= math.sin(a) / a
        out = np.fft.irfft(fk, n=size)
        for p_ in range(nd):
            flat[idx[p_]] = out[p_ + pad]
    return flat.reshape(nd, n)


def natural_cspline(x, y):
    """Second derivatives M of the natural cubic spline through (x, y)."""
    n = len(x)
    mm = np.zeros(n)
    if n < 3:
        return mm
    h = np.diff(x)
    k = n - 2
    diag = 2.0 * (h[:-1] + h[1:])
    upper = h[1:].copy()
    rhs = 6.0 * ((y[2:] - y[1:-1]) / h[1:] - (y[1:-1] - y[:-2]) / h[:-1])
    for j in range(1, k):
        f = h[j] / diag[j - 1]
        diag[j] -= f * upper[j - 1]
        rhs[j] -= f * rhs[j - 1]
    mm[k] = rhs[k - 1] / diag[k - 1]
    for j in range(k - 2, -1, -1):
        mm[j + 1] = (rhs[j] - upper[j] * mm[j + 2]) / diag[j]
    return mm


def cspline_eval(x, y, mm, t):
    """Natural cubic spline at t (x[0] <= t <= x[-1])."""
    i = min(max(int(np.searchsorted(x, t, side="right")) - 1, 0), len(x) - 2)
    h = x[i + 1] - x[i]
    t1, t0 = x[i + 1] - t, t - x[i]
    return ((mm[i] * t1 ** 3 + mm[i + 1] * t0 ** 3) / (6.0 * h)
            + (y[i] / h - mm[i] * h / 6.0) * t1 + (y[i + 1] / h - mm[i + 1] * h / 6.0) * t0)


def cspline_slope(x, y, mm, i, t):
    """First derivative at t of the natural cubic spline's piece on [x_i, x_{i+1}]."""
    h = x[i + 1] - x[i]
    t1, t0 = x[i + 1] - t, t - x[i]
    return ((3.0 * mm[i + 1] * t0 * t0 - 3.0 * mm[i] * t1 * t1) / (6.0 * h)
            - (y[i] / h - mm[i] * h / 6.0) + (y[i + 1] / h - mm[i + 1] * h / 6.0))


def flux_conversion(settings):
    """conv::readConversion's resolution of InputIsDeltaFlux, UseChunksMeanFlux
    and MeanFluxFile (core/fiducial_cosmology.cpp:33-83): delta input wins, then
    the spectrum's own mean, then the file; 'none', 'mean' or 'file'."""
    if settings is None or settings.input_is_delta_flux:
        return "none"
    if settings.use_chunks_mean_flux:
        return "mean"
    if settings.mean_flux is not None:
        return "file"
    return "none"


def mean_flux_at(mean_flux, z):
    """F-bar(z): Interpolation::evaluate with GSL_CUBIC_INTERPOLATION
    (mathtools/interpolation.cpp:42-62), the natural cubic spline and, past
    either end, the line along its end slope."""
    x, y = (np.asarray(a, dtype=np.float64) for a in mean_flux)
    mm = natural_cspline(x, y)
    if z < x[0]:
        return cspline_eval(x, y, mm, x[0]) + (z - x[0]) * cspline_slope(x, y, mm, 0, x[0])
    if z > x[-1]:
        n = len(x)
        return cspline_eval(x, y, mm, x[-1]) + (z - x[-1]) * cspline_slope(x, y, mm, n - 2, x[-1])
    return cspline_eval(x, y, mm, z)


def convert_flux_to_delta(settings, wave, flux, ivar):
    """conv::chunkMeanConversion / fullConversion (core/fiducial_cosmology.cpp:94-111)
    on a whole spectrum, in place: delta = F / F-bar - 1, ivar F-bar^2, F-bar
    the mean over every pixel (masked ones too, summed in order) or F-bar(z)."""
    kind = flux_conversion(settings)
    if kind == "mean":
        mean = float(np.add.accumulate(flux)[-1]) / len(flux)
        flux[:] = flux / mean - 1
        ivar *= mean * mean
    elif kind == "file":
        for i in range(len(flux)):
            fbar = mean_flux_at(settings.mean_flux, wave[i] / LYA_REST - 1)
            flux[i] = flux[i] / fbar - 1
            ivar[i] *= fbar * fbar


def _nonzero_min_element(row):
    """nonzero_min_element, mathtools/matrix_helper.cpp:20-39."""
    smallest = abs(row[0])
    for v in row[1:]:
        tmp = abs(v)
        if smallest < 1e-15:
            smallest = tmp
        elif tmp < smallest and tmp > 1e-15:
            smallest = tmp
    return max(smallest, 1e-15)


def dia_oversample(values, osamp, dlambda):
    """Resolution::oversample, mathtools/matrix_helper.cpp:1008-1073: each row's
    ndiags entries, shifted positive and log-transformed, go through a natural
    cubic spline evaluated at osamp x finer spacing; rows renormalised to unit
    sum.  Returns rows [n][2 noff osamp + 1]."""
    nd, n = values.shape
    flat = values.ravel()
    noff = nd // 2
    nelem = 2 * noff * osamp + 1
    win = np.array([(i - noff) * dlambda for i in range(nd)])
    wout = np.array([(i * 1. / osamp - noff) * dlambda for i in range(nelem)])
    out = np.empty((n, nelem))
    for i in range(n):
        row = flat[dia_row_indices(i, n, nd)].copy()
        shift = float(np.min(row)) - _nonzero_min_element(row)
        lrow = np.log(row - shift)
        mm = natural_cspline(win, lrow)
        new = np.array([shift + math.exp(cspline_eval(win, lrow, mm, t)) for t in wout])
        out[i] = new * (1.0 / new.sum())
    return out


def resolution_dense(rows, oversampled, n):
    """Dense R of a chunk: oversampled rows (n x nelem) sit at columns
    i * osamp .. (OversampledMatrix, matrix_helper.cpp:859-920); a diagonal
    matrix values[ndiags][n] gives R[c - off][c] = values[d][c]."""
    if oversampled is not None:
        nelem = rows.shape[1]
        ncols = n * oversampled + nelem - 1
        r = np.zeros((n, ncols))
        for i in range(n):
            r[i, i * oversampled:i * oversampled + nelem] = rows[i]
        return r
    nd = rows.shape[0]
    noff = nd // 2
    r = np.zeros((n, n))
    for d in range(nd):
        off = noff - d
        for c in range(n):
            row = c - off
            if 0 <= row < n:
                r[row, c] = rows[d, c]
    return r


def decide_indices(wave, settings):
    """OneQSOEstimate::decideIndices, core/one_qso_estimate.cpp:17-50."""
    vel = C_KMS * np.log(wave / wave[0])
    vmax = vel[-1]
    nchunks = 1
    if settings.number_of_chunks > 1:
        nchunks += int(vmax / settings.max_forest_length_v)
        vmax = min(settings.max_forest_length_v, vmax / nchunks)
    idx = [0]
    vl = 0
    vel = vel.copy()
    for _ in range(nchunks):
        jj = vl + int(np.searchsorted(vel[vl:], vmax, side="right"))
        idx.append(jj)
        if jj == len(wave):
            break
        vl = jj
        vel[vl:] -= vel[vl]
    return idx


def make_chunk(wave, delta, ivar, r_fwhm, bins, table_keys, settings, reso=None, rm=None):
    """Chunk::Chunk, core/chunk_estimate.cpp:141-257 (raises ValueError where
    the reference throws).  table_keys maps (R, dv rounded to 0.1) -> index.
    With a resolution matrix (reso = (oversampling, m), rm its slice for these
    pixels) the table is the first one (RES_INDEX = 0, :189-193)."""
    a, b = cut_masked_boundary(ivar)
    wave, delta, ivar = wave[a:b].copy(), delta[a:b].copy(), ivar[a:b].copy()
    if rm is not None:
        rm = rm[a:b] if reso[0] > 0 else rm[:, a:b]
    n = len(wave)
    realsize = int((ivar != 0).sum())
    dv = _median(np.log(wave[1:] / wave[:-1]) * C_KMS) if n > 1 else -1.0
    lenv = C_KMS * math.log(wave[-1] / wave[0]) if n else 0.0
    minnopix = int(lenv / settings.max_pixel_length_v)
    if realsize < minnopix or lenv < settings.min_forest_length_v:
        raise ValueError("Short chunk")
    rounded = _c_round(dv * 10) / 10
    res_index = -1
    if reso is not None:
        res_index = 0
    for (r, tdv), idx in table_keys.items():
        if res_index >= 0:
            break
        if r == r_fwhm and abs(rounded - tdv) < 0.01:
            res_index = idx
            break
    if res_index < 0:
        raise KeyError(f"SpecRes R: {r_fwhm}, dv: {dv} not found in tables!")
    zmin, zmax = wave[0] / LYA_REST - 1, wave[-1] / LYA_REST - 1
    kbin_upp = int(np.searchsorted(bins.k_centers, 0.85 * (math.pi / dv), side="left"))
    zlow, zupp = find_redshift_bin(bins, zmin), find_redshift_bin(bins, zmax)
    nq = zupp - zlow + 1
    fis = zlow * bins.nk
    if bins.triangular:
        if zmin < bins.z_centers[zlow] and zlow != 0:
            nq += 1
            fis -= bins.nk
        if bins.z_centers[zupp] < zmax and zupp < bins.nz - 1:
            nq += 1
    nq *= bins.nk
    rmat = fine = None
    if reso is not None:
        osamp = reso[0]
        # sparse (banded) R: R M R^T costs O(n^2 nelem) as in the reference
        rmat = sparse.csr_matrix(resolution_dense(rm, osamp if osamp > 0 else None, n))
        w0 = wave[0] / LYA_REST
        if osamp > 0:
            # Chunk::_initMatrices, core/chunk_estimate.cpp:927-938; dlambda is
            # the chunk's median pixel width (QSOFile copy, io/qso_file.cpp:86-88)
            dlam = _median(np.diff(wave)) if n > 1 else -1.0
            fine_dl = dlam / LYA_REST / osamp
            disp = rm.shape[1] // 2
            fine = np.array([w0 + (i - disp) * fine_dl for i in range(rmat.shape[1])])
        else:
            fine = wave / LYA_REST
    return ChunkData(wave / LYA_REST, delta, ivar, int(r_fwhm), float(dv), res_index, kbin_upp,
                     zlow, zupp, nq, fis, rmat, fine)


def chunks_from_spectra(spectra, bins, table_keys, settings, reso=None):
    """OneQSOEstimate construction for every spectrum; chunks the reference
    would reject are skipped, as OneQSOEstimate::OneQSOEstimate does.
    reso = (oversampling, deconvolution m) uses each spectrum's resolution
    matrix (UseResoMatrix)."""
    out = []
    for s in spectra:
        try:
            pre = preprocess_spectrum(s, bins, reso, settings)
        except ValueError:
            continue
        wave, delta, ivar = pre[:3]
        rm = pre[3] if reso is not None else None
        idx = decide_indices(wave, settings)
        for i1, i2 in zip(idx[:-1], idx[1:]):
            sl = None
            if rm is not None:
                sl = rm[i1:i2] if reso[0] > 0 else rm[:, i1:i2]
            try:
                out.append(make_chunk(wave[i1:i2], delta[i1:i2], ivar[i1:i2], s.r_fwhm, bins,
                                      table_keys, settings, reso, sl))
            except (ValueError, KeyError):
                continue
    return out


# ---------------------------------------------------------------------------
# Per-chunk QMLE (core/chunk_estimate.cpp:384-914)

def interp1d(y, x1, dx, x):
    """DiscreteInterpolation1D::evaluate, mathtools/discrete_interpolation.cpp:61-72."""
    xx = (x - x1) / dx
    n = np.trunc(xx).astype(np.int64)
    n = np.clip(n, 0, len(y) - 2)
    dn = xx - n
    return y[n] * (1 - dn) + y[n + 1] * dn


def interp2d(zarr, nx, ny, x1, dx, y1, dy, x, y):
    """DiscreteInterpolation2D::evaluate, mathtools/discrete_interpolation.cpp:221-242;
    zarr is flat with x fastest (index nx + Nx * ny)."""
    xx, yy = (x - x1) / dx, (y - y1) / dy
    ix = np.clip(np.trunc(xx).astype(np.int64), 0, nx - 2)
    iy = np.clip(np.trunc(yy).astype(np.int64), 0, ny - 2)
    ind = ix + nx * iy
    dnx, dny = xx - ix, yy - iy
    return (zarr[ind] * (1 - dnx) * (1 - dny) + zarr[ind + 1] * dnx * (1 - dny)
            + zarr[ind + nx] * (1 - dnx) * dny + zarr[ind + nx + 1] * dnx * dny)


def zbin_weight(bins, zm, z):
    """Redshift weights of bin zm, element-wise form of
    core/global_numbers.cpp:393-471 (the reference applies them along sorted
    rows; on a sorted row these conditions select the same elements)."""
    zc, dz = bins.z_centers[zm], bins.dz
    out = np.zeros_like(z)
    if (not bins.triangular) or bins.nz == 1:
        out[(z >= zc - dz / 2) & (z <= zc + dz / 2)] = 1.0
        return out
    inside = (z >= zc - dz) & (z <= zc + dz)
    out[inside] = 1.0 - np.abs(z[inside] - zc) / dz
    if zm == 0:
        out[z < zc] = 1.0
    if zm == bins.nz - 1:
        out[z > zc] = 1.0
    return out


SMOOTH_HWSIZE = 25                # Smoother::HWSIZE (mathtools/smoother.hpp:12)


def _median_statistics(arr, thres=1e3):
    """_findMedianStatistics (mathtools/smoother.cpp:66-81): median, mean and
    scaled MAD of the sorted values <= thres (the mean a sequential sum)."""
    a = np.sort(arr)
    m = len(a)
    while m and a[m - 1] > thres:
        m -= 1
    if m == 0:
        return a[0], math.nan, math.nan
    median = _median_sorted(a[:m])
    mean = float(np.cumsum(a[:m])[-1]) / m
    mad = 1.4826 * _median_sorted(np.sort(np.abs(a[:m] - median)))
    return median, mean, mad


def smooth_ivar(ivar, sigmapix):
    """Smoother::smoothIvar (mathtools/smoother.cpp:171-217) with its filter
    (_constructFilter :102-113), padding (padArray :18-26: the right-hand pad
    is written over the last SMOOTH_HWSIZE pixels, the cells past them stay 0)
    and masked-region fill (_fillMaskedRegion :84-99)."""
    ivar = np.asarray(ivar, dtype=np.float64)
    n, hw = len(ivar), SMOOTH_HWSIZE
    with np.errstate(divide="ignore"):
        var = np.where(ivar == 0, 1e15, 1.0 / ivar)
    median, mean, mad = _median_statistics(var)
    if math.isnan(mean):
        return ivar.copy()
    mean = 1.0 / mean
    cut = 1.0 / (median + 3.5 * mad)
    masked = np.flatnonzero(ivar < cut)
    if sigmapix == 0:
        out = np.full(n, mean)
    else:
        pad = np.zeros(n + 2 * hw)
        pad[hw:hw + n] = ivar
        pad[:hw] = ivar[0]
        pad[n:n + hw] = ivar[-1]
        if masked.size:
            if masked[0] == 0:
                pad[:hw] = mean
            pad[masked + hw] = mean
            if masked[-1] == n - 1:
                pad[-hw:] = mean
        with np.errstate(divide="ignore"):
            pad = 1.0 / pad
        x = np.arange(-hw, hw + 1) * 1.0 / sigmapix
        g = np.exp(-(x * x) / 2)
        g = g / float(np.cumsum(g)[-1])
        win = np.lib.stride_tricks.sliding_window_view(pad, 2 * hw + 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            out = 1.0 / (win @ g)
    out[masked] = ivar[masked]
    return out


def smooth_rows(values, sigmapix):
    """Smoother::smooth1D (mathtools/smoother.cpp:144-168) on every row of
    values (a DiaMatrix's diagonals): sigmapix = 0 the mean of the row's values
    <= 1e3, else the 51-tap Gaussian convolution after padArray's padding."""
    out = np.array(values, dtype=np.float64)
    hw = SMOOTH_HWSIZE
    x = np.arange(-hw, hw + 1) * 1.0 / max(sigmapix, 1)
    g = np.exp(-(x * x) / 2)
    g = g / float(np.cumsum(g)[-1])
    for r in range(out.shape[0]):
        row = out[r]
        n = len(row)
        if sigmapix == 0:
            a = np.sort(row)
            m = len(a)
            while m and a[m - 1] > 1e3:
                m -= 1
            out[r] = float(np.cumsum(a[:m])[-1]) / m
            continue
        pad = np.zeros(n + 2 * hw)
        pad[hw:hw + n] = row
        pad[:hw] = row[0]
        pad[n:n + hw] = row[-1]
        out[r] = np.lib.stride_tricks.sliding_window_view(pad, 2 * hw + 1) @ g
    return out


def _sym_upper(a):
    return np.triu(a) + np.triu(a, 1).T


def lu_inverse(a):
    """LAPACKE_InvertMatrixLU, mathtools/matrix_helper.cpp:184-204."""
    lu, piv, info = lapack.dgetrf(a)
    if info != 0:
        raise np.linalg.LinAlgError("ERROR in LU decomposition.")
    inv, info = lapack.dgetri(lu, piv)
    if info != 0:
        raise np.linalg.LinAlgError("ERROR in LU invert.")
    return inv


@dataclasses.dataclass
class TableView:
    """The interpolation grids SQLookupTable builds (core/sq_table.cpp:148-175, 325-368)."""
    deriv: np.ndarray      # nk x nv
    signal: np.ndarray     # nv x nz (z fastest)
    v1: float
    dv: float
    z1: float
    dz: float


def table_view(table, bins, nv, lenv, nzp):
    lenz = bins.dz * (bins.nz + 1)
    return TableView(np.asarray(table.deriv), np.asarray(table.signal), 0.0, lenv / (nv - 1.0),
                     bins.z_centers[0] - bins.dz, lenz / (nzp - 1.0))


def build_matrices(ch: ChunkData, bins, tv: TableView, growth_b=None):
    """v/z matrices, stored Q_k with redshift weights, and S_fid
    (core/chunk_estimate.cpp:384-536, :861-882).  Returns (stored i_kz list,
    Q stack [ns, n, n], S).  growth_b: RedshiftGrowthOn with exponent B
    (_scaleDerivativesWithRedshiftGrowth, :539-573), Q_k of bin m times
    ((1 + z_ij) / (1 + z_m))^B, on the full symmetric z_ij (the reference's
    z matrix is only complete with an oversampled resolution matrix; without
    one its lower triangle is scratch that the growth step reads as it is)."""
    n = ch.n
    li, lj = ch.wave[:, None], ch.wave[None, :]
    vmat = C_KMS * np.log(lj / li)
    zmat = np.sqrt(li * lj) - 1.0
    iu = np.triu_indices(n)
    stored = [i for i in range(ch.nq) if (i + ch.fisher_index_start) % bins.nk < ch.kbin_upp]
    ns = len(stored)
    q = np.empty((ns, n, n))
    vu = vmat[iu]
    nzp = tv.signal.shape[1]
    if ch.rmat is None:
        for kn in range(ch.kbin_upp):
            m = np.empty((n, n))
            m[iu] = interp1d(tv.deriv[kn], tv.v1, tv.dv, vu)
            q[kn] = _sym_upper_fill(m)
        sm = np.empty((n, n))
        sm[iu] = interp2d(tv.signal.ravel(), nzp, tv.signal.shape[0], tv.z1, tv.dz, tv.v1, tv.dv,
                          zmat[iu], vu)
        sm = _sym_upper_fill(sm)
    else:
        # UseResoMatrix: S and Q_k on the resolution matrix's grid, then
        # R . M . R^T (core/chunk_estimate.cpp:400-480); Q_k is the analytic
        # band (dk / pi) cos(k_c v) sinc(dk v / 2) (:444-454)
        nf = len(ch.fine_wave)
        fi, fj = ch.fine_wave[:, None], ch.fine_wave[None, :]
        iuf = np.triu_indices(nf)
        vf = (C_KMS * np.log(fj / fi))[iuf]
        zf = (np.sqrt(fi * fj) - 1.0)[iuf]
        r = ch.rmat
        for kn in range(ch.kbin_upp):
            kc = bins.k_centers[kn]
            dk = bins.k_edges[kn + 1] - bins.k_edges[kn]
            x = dk * vf / 2
            with np.errstate(invalid="ignore", divide="ignore"):
                val = np.where(vf == 0, dk / math.pi, (dk / math.pi) * np.cos(kc * vf) * (np.sin(x) / x))
            m = np.empty((nf, nf))
            m[iuf] = val
            m = _sym_upper_fill(m)
            q[kn] = _sym_upper_fill(np.asarray((r @ m) @ r.T))
        m = np.empty((nf, nf))
        m[iuf] = interp2d(tv.signal.ravel(), nzp, tv.signal.shape[0], tv.z1, tv.dz, tv.v1, tv.dv,
                          zf, vf)
        m = _sym_upper_fill(m)
        sm = _sym_upper_fill(np.asarray((r @ m) @ r.T))
    for s in range(ch.kbin_upp, ns):
        q[s] = q[stored[s] % bins.nk]
    zu = zmat[iu]
    nzb = ns // ch.kbin_upp
    for iz in range(nzb):
        zm = ch.fisher_index_start // bins.nk + iz
        w = np.zeros((n, n))
        w[iu] = zbin_weight(bins, zm, zu)
        w = _sym_upper_fill(w)
        q[iz * ch.kbin_upp:(iz + 1) * ch.kbin_upp] *= w[None]
    if growth_b is not None:
        z1 = zmat + 1.0
        for iz in range(nzb):
            zm = ch.fisher_index_start // bins.nk + iz
            g = (z1 / (bins.z_centers[zm] + 1)) ** growth_b
            q[iz * ch.kbin_upp:(iz + 1) * ch.kbin_upp] *= g[None]
    return stored, q, sm


def _sym_upper_fill(m):
    """mxhelp::copyUpperToLower (mathtools/matrix_helper.cpp:81-94)."""
    il = np.tril_indices(m.shape[0], -1)
    m[il] = m.T[il]
    return m


def inverse_covariance(ch: ChunkData, stored, q, sm, theta, settings):
    """Chunk::setInvertCovarianceMatrix, core/chunk_estimate.cpp:668-719, with
    _addMarginalizations :576-665."""
    n = ch.n
    cov = np.zeros((n, n)) if settings.turn_off_sfid else sm.copy()
    for s, ikz in enumerate(stored):
        cov += theta[ch.fisher_index_start + ikz] * q[s]
    ivec = ch.ivar
    if settings.smooth_noise_weights >= 0:
        ivec = smooth_ivar(ch.ivar, settings.smooth_noise_weights)
    cov *= ivec[:, None]
    cov[np.diag_indices(n)] += 1.0
    cinv = lu_inverse(cov)
    cinv *= ivec[None, :]
    nvec = settings.cont_nvecs
    if nvec > 0:
        vecs = [np.full(n, 1.0 / math.sqrt(n))]
        for cmo in range(1, settings.cont_logl_order + 1):
            v = np.log(ch.wave) ** cmo
            vecs.append(v * (1.0 / np.linalg.norm(v)))
        for cmo in range(1, settings.cont_l_order + 1):
            v = ch.wave ** cmo
            vecs.append(v * (1.0 / np.linalg.norm(v)))
        a = np.stack(vecs, axis=1)                 # n x nvec, column-major view of marg_mat
        u, svals, _vt, info = lapack.dgesvd(a, compute_uv=1, full_matrices=0)
        if info != 0:
            raise np.linalg.LinAlgError("ERROR in SVD.")
        nuse = nvec
        while nuse > 0 and not (svals[nuse - 1] / svals[0] > DOUBLE_EPSILON):
            nuse -= 1
        for i in range(nuse):
            v = u[:, i]
            y = _sym_upper(cinv) @ v
            norm = -1.0 / np.dot(v, y)
            cinv += norm * np.outer(y, y)
    return cinv


def chunk_iteration(ch: ChunkData, bins, tv: TableView, theta, settings, compute_fisher=True):
    """Chunk::oneQSOiteration for one chunk: returns (d, b, t, F) with
    F (nq x nq) upper triangle filled and not halved (core/chunk_estimate.cpp:738-914)."""
    stored, q, sm = build_matrices(ch, bins, tv, settings.growth_b if settings.redshift_growth else None)
    cinv = inverse_covariance(ch, stored, q, sm, theta, settings)
    n, nq, ns = ch.n, ch.nq, len(stored)
    d, b, t = np.zeros(nq), np.zeros(nq), np.zeros(nq)
    y = _sym_upper(cinv) @ ch.delta
    for s, ikz in enumerate(stored):
        d[ikz] = y @ (_sym_upper(q[s]) @ y)
    a = np.matmul(cinv[None], q)                   # C^-1 Q_k, :721-736
    wn = np.zeros((n, n))
    good = ch.ivar != 0
    wn[good] = (1.0 / ch.ivar[good])[:, None] * cinv[good]
    a2 = a.reshape(ns, -1)
    b[stored] = a2 @ wn.ravel()
    if not settings.turn_off_sfid:
        ws = sm @ cinv
        t[stored] = a2 @ ws.ravel()
    fisher = np.zeros((nq, nq))
    if compute_fisher:
        at = np.ascontiguousarray(a.transpose(0, 2, 1)).reshape(ns, -1)
        f = at @ a2.T                              # F_ij = <A_i^T, A_j>
        idx = np.array(stored)
        fu = np.triu(f)
        if settings.fisher_optimization:
            # only the bands |j - i| <= 5 and |j - i - Nk| <= 2 of the local kz
            # indices are computed, the rest stays 0 (core/chunk_estimate.cpp:823-827)
            diff = idx[None, :] - idx[:, None]
            fu = np.where((diff > 5) & (np.abs(diff - bins.nk) > 2), 0.0, fu)
        fisher[np.ix_(idx, idx)] = fu
    return d, b, t, fisher


# ---------------------------------------------------------------------------
# Global step (core/quadratic_estimate.cpp:456-457, 261-318;
# mathtools/matrix_helper.cpp:220-358)

def accumulate(nkz, results):
    """Sum per-chunk (fisher_index_start, d, b, t, F) into the global arrays
    (core/chunk_estimate.cpp:893-903)."""
    fsum = np.zeros((nkz, nkz))
    dbt = np.zeros((3, nkz))
    for fis, d, b, t, f in results:
        nq = len(d)
        fsum[fis:fis + nq, fis:fis + nq] += np.triu(f)
        dbt[0, fis:fis + nq] += d
        dbt[1, fis:fis + nq] += b
        dbt[2, fis:fis + nq] += t
    return fsum, dbt


def stable_invert_sym(s):
    """mxhelp::stableInvertSym: returns (solver matrix, inverse, warn, dof, damp)."""
    s = s.copy()
    nkz = s.shape[0]
    empty = [i for i in range(nkz) if s[i, i] == 0]
    for i in empty:
        s[i, i] = 1.0
    svals = lapack.dgesvd(s.copy(), compute_uv=0)[1]
    damp = 0.0
    for i in range(nkz - 1, 0, -1):
        if svals[i - 1] / svals[i] > 8.0:
            damp = svals[i]
        else:
            break
    if damp != 0:
        sinv = lu_inverse(s.copy())
        amat = s @ s
        amat[np.diag_indices(nkz)] += damp
        solver = lu_inverse(amat) @ s
        warn = 1
    else:
        solver = lu_inverse(s.copy())
        sinv = solver.copy()
        warn = 0
    for i in empty:
        solver[i, i] = 0.0
        sinv[i, i] = 0.0
    return solver, sinv, warn, nkz - len(empty), damp


def newton_raphson_step(fsum, dbt):
    """F *= 1/2, symmetrise, invert, theta = 1/2 F^-1 (d - b - t)."""
    f = 0.5 * fsum
    f = _sym_upper_fill(f)
    solver, sinv, warn, dof, damp = stable_invert_sym(f)
    w = 0.5 * (solver @ dbt.T).T
    theta = w[0] - w[1] - w[2]
    return dict(fisher=f, solver=solver, inverse=sinv, theta=theta, warn=warn, dof=dof, damp=damp,
                weighted=w)


# ---------------------------------------------------------------------------
# Complete bootstrap (FastBootstrap 0): core/bootstrapper.hpp:126-135,
# 217-257, 291-345, core/one_qso_estimate.cpp:200-238, one_qso_estimate.hpp:43-53

def complete_bootstrap(nkz, chunks, qso_offsets, p):
    """chunks: per batch chunk (fisher_index_start, nq, d, b, t, F upper);
    qso_offsets: spectrum q owns chunks [off[q], off[q+1]); p[q, b]: the
    coefficient of spectrum q in realization b.  Returns (slots, n_valid,
    mean, cov) as PoissonBootstrapper leaves them."""
    from scipy.linalg import cho_factor, cho_solve
    nq_, nb = p.shape
    blocks = []
    for q in range(nq_):
        cs = chunks[qso_offsets[q]:qso_offsets[q + 1]]
        if not cs:
            blocks.append((0, np.zeros(0), np.zeros((0, 0))))
            continue
        lo = min(c[0] for c in cs)
        hi = max(c[0] + c[1] for c in cs)
        th, fq = np.zeros(hi - lo), np.zeros((hi - lo, hi - lo))
        for fis, nq, d, b, t, f in cs:
            o = fis - lo
            th[o:o + nq] += (d - b) - t
            fq[o:o + nq, o:o + nq] += np.triu(f)
        blocks.append((lo, th, fq))
    slots = np.zeros((nb, nkz))
    nvalid = 0
    for jj in range(nb):
        power, fisher = np.zeros(nkz), np.zeros((nkz, nkz))
        for q, (lo, th, fq) in enumerate(blocks):
            if p[q, jj] == 0:
                continue
            m = len(th)
            fisher[lo:lo + m, lo:lo + m] += p[q, jj] * fq
            power[lo:lo + m] += p[q, jj] * th
        slots[nvalid] = power
        empty = np.flatnonzero(np.diag(fisher) == 0)
        fisher[empty, empty] = 1.0
        full = np.triu(fisher) + np.triu(fisher, 1).T
        try:
            x = cho_solve(cho_factor(full, lower=False), power)
        except np.linalg.LinAlgError:
            continue
        x[empty] = 0.0
        slots[nvalid] = x
        nvalid += 1
    mean = np.cumsum(slots, axis=0)[-1] * (1.0 / nvalid)
    v = slots - mean
    cov = (v.T @ v) * (1.0 / (nvalid - 1))
    return slots, nvalid, mean, cov
