"""Smoothing step of lyspeq's Newton-Raphson loop as a command, with the
interface of lyspeq's py/smbivspline.py, which
OneDQuadraticPowerEstimate::_smoothPowerSpectra runs between iterations
(core/quadratic_estimate.cpp:353-396):

    python -m lyspeq_gb300.smoothing InputPS OutputPS [--interp_log]

InputPS is the estimate as writeSpectrumEstimates prints it (a line "Nz Nk",
a line of counts, then "z k P e" per bin); OutputPS receives the smoothed P,
one value per line, in the same order.  The fit is
lyspeq_gb300.estimator.smooth_power (scipy's SmoothBivariateSpline with the
script's weights and smoothing factor)."""
from __future__ import annotations

import argparse

import numpy as np

from .estimator import smooth_power


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("InputPS")
    ap.add_argument("OutputPS")
    ap.add_argument("--interp_log", action="store_true")
    args = ap.parse_args(argv)
    z, k, p, e = np.genfromtxt(args.InputPS, delimiter=" ", skip_header=2, unpack=True)
    np.savetxt(args.OutputPS, smooth_power(z, k, p, e, args.interp_log), header="", comments="")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
