"""Newton-Raphson loop of lyspeq's estimator on the GPU engine.

Host-side mirror of ``OneDQuadraticPowerEstimate::iterate``
(core/quadratic_estimate.cpp:398-546): each iteration runs one batched
``lqg_nr_iteration`` with the current power-spectrum fit, inverts the global
Fisher matrix (``lqg_fisher_solve``: ``invertTotalFisherMatrix`` and
``computePowerSpectrumEstimates``, :261-318), tests convergence
(``hasConverged``, :548-614) and, unless done, smooths the estimate as the
reference's ``_smoothPowerSpectra`` (:353-396) does with its script
py/smbivspline.py: the estimate is written as text (``writeSpectrumEstimates``,
:624-652, so with seven significant digits), fitted by a weighted smoothing
bivariate spline (scipy's ``SmoothBivariateSpline``, the library that script
calls) and read back as the next iteration's fit minus the fiducial power.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import synth


def smooth_power(z, k, p, e, interp_log=False):
    """The smoothing of py/smbivspline.py: a smoothing bivariate spline in
    (z, k) through P with weights 1/e and smoothing factor len(e); with
    interp_log, in (ln(1+z), ln k, ln P) through the points with P, e > 0 and
    weights P/e."""
    from scipy.interpolate import SmoothBivariateSpline
    z, k, p, e = (np.asarray(a, dtype=np.float64) for a in (z, k, p, e))
    if interp_log:
        mask = (p > 0) & (e > 0)
        lnz, lnk, lnp = np.log(1 + z[mask]), np.log(k[mask]), np.log(p[mask])
        lne = e[mask] / p[mask]
        spl = SmoothBivariateSpline(lnz, lnk, lnp, w=1. / lne, s=len(lne))
        return np.exp(spl(np.log(1 + z), np.log(k), grid=False))
    spl = SmoothBivariateSpline(z, k, p, w=1. / e, s=len(e))
    return spl(z, k, grid=False)


def spectrum_rows(bins, theta, inverse, pfid):
    """(z, k, P, e) as writeSpectrumEstimates prints them ("%.3lf %e %e %e")
    and the smoothing script reads them back."""
    rows = []
    nk = bins.nk
    for ikz in range(bins.nkz):
        zm, kn = divmod(ikz, nk)
        p = theta[ikz] + pfid[ikz]
        e = math.sqrt(inverse[ikz, ikz])
        rows.append(tuple(float(x) for x in ("%.3f %e %e %e" % (bins.z_centers[zm], bins.k_centers[kn], p, e)).split()))
    return np.array(rows)


def has_converged(current, previous, inverse, fisher, dof, eps):
    """OneDQuadraticPowerEstimate::hasConverged: with dp = previous - current,
    converged when sqrt(sum dp^2 / diag(F^-1) / dof) < eps or
    sqrt(|dp^T F dp| / dof) < eps.  Returns (converged, dp)."""
    dp = previous - current
    e = np.diag(inverse)
    ok = e > 0
    r = math.sqrt(float(np.sum(dp[ok] ** 2 / e[ok])) / dof)
    rfull = math.sqrt(abs(float(dp @ (fisher @ dp))) / dof)
    return (r < eps or rfull < eps), dp


@dataclasses.dataclass
class NRResult:
    theta: np.ndarray            # final estimate (current_power_estimate_vector)
    previous: np.ndarray         # previous estimate minus the final one (as hasConverged leaves it)
    fits: np.ndarray             # the smoothed fit the last iteration used (powerspectra_fits)
    fisher: np.ndarray           # global Fisher matrix, halved and symmetric
    inverse: np.ndarray
    solver: np.ndarray
    dbt: np.ndarray              # 3 x nkz sums before Fisher weighting
    iterations: int
    converged: bool


class QuadraticEstimator:
    """OneDQuadraticPowerEstimate on an lqg.Engine whose batch holds the chunks.

    number_of_iterations, chisq_eps and smooth_log are the NumberOfIterations,
    ChiSqConvergence and SmoothLnkLnP settings; fid the fiducial PD13
    parameters; turn_off_sfid TurnOffBaseline (no fiducial power, as the
    engine's C has no fiducial signal); precomputed_fisher the matrix of a
    PrecomputedFisher file (halved, nkz x nkz), used in place of the chunks'
    sum (core/quadratic_estimate.cpp:478-483; the engine then needs
    skip_fisher)."""

    def __init__(self, engine, bins, fid=synth.PD13_DEFAULT, number_of_iterations=1, chisq_eps=0.01,
                 smooth_log=False, precision="fp64", turn_off_sfid=False, precomputed_fisher=None):
        self.engine, self.bins = engine, bins
        self.iterations = int(number_of_iterations)
        self.eps = float(chisq_eps)
        self.smooth_log = bool(smooth_log)
        self.precision = precision
        # powerSpectrumFiducial(kn, zm) for every bin (i_kz = zm nk + kn); 0
        # with TurnOffBaseline (core/quadratic_estimate.cpp, powerSpectrumFiducial)
        self.pfid = synth.pd13_power(np.tile(bins.k_centers, bins.nz), np.repeat(bins.z_centers, bins.nk), fid)
        if turn_off_sfid:
            self.pfid = np.zeros_like(self.pfid)
        self.precomputed = None
        if precomputed_fisher is not None:
            self.precomputed = np.asarray(precomputed_fisher, dtype=np.float64)
            if self.precomputed.shape != (bins.nkz, bins.nkz):
                raise ValueError("Precomputed Fisher matrix does not have correct number of rows or columns.")

    def iterate(self) -> NRResult:
        nkz = self.bins.nkz
        fits = np.zeros(nkz)
        current = np.zeros(nkz)
        converged = False
        it = 0
        for it in range(1, self.iterations + 1):
            self.engine.iterate(theta=fits, precision=self.precision)
            out = self.engine.download()
            dbt = np.stack([out["d"], out["b"], out["t"]])
            # the solve takes the unhalved sum: twice the halved matrix, exactly
            fsum = out["fisher"] if self.precomputed is None else 2.0 * self.precomputed
            g = self.engine.fisher_solve(fsum, dbt)
            previous, current = current, g["theta"]
            converged, previous = has_converged(current, previous, g["inverse"], g["fisher"], g["dof"], self.eps)
            if converged or it == self.iterations:
                break
            rows = spectrum_rows(self.bins, current, g["inverse"], self.pfid)
            fits = smooth_power(rows[:, 0], rows[:, 1], rows[:, 2], rows[:, 3], self.smooth_log) - self.pfid
        return NRResult(current, previous, fits, g["fisher"], g["inverse"], g["solver"], dbt, it, converged)
