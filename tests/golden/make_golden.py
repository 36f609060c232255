"""Generate the golden fixtures of the parity tests.

Each fixture holds a seeded synthetic workload (binning, lookup-table keys
and the chunks exactly as lyspeq hands them to Chunk::oneQSOiteration; the
tables themselves are rebuilt by lyspeq_gb300.synth.build_table) together
with the outputs of lyspeq itself on those inputs: per-chunk d, b, t and
Fisher matrices and the global Newton-Raphson results.  The outputs come from
the reference compiled from its own sources (oracle/refbuild, run through
oracle/_ref/chunk_driver with one OpenMP thread), so the fixtures travel to
machines where the reference sources are absent.

Fixture lyspeq_test_it1 holds lyspeq's own end-to-end test input and truth
(read from the lyspeq tree, see make_lyspeq_test).

Run (needs the oracle built: make -C oracle/refbuild):
    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lyspeq_gb300 import synth  # noqa: E402
from oracle import refdump  # noqa: E402

LYA_REST = synth.LYA_REST

# name -> (workload, n_chunks, (logl, lam) marginalisation orders, masked-pixel fraction,
#          chunks kept in the fixture)
CASES = {
    "tiny_nomarg": ("tiny", None, (-1, -1), 0.0, None),
    "tiny_marg1": ("tiny", None, (1, -1), 0.0, None),
    "tiny_marg3": ("tiny", None, (2, 1), 0.0, None),
    "tiny_masked": ("tiny", None, (1, -1), 0.04, None),
    "small_cfg": ("small", None, (-1, -1), 0.0, 12),
    "desi_sub": ("desi", 6, (1, -1), 0.0, None),
    # echelle-size chunks: N 1000-1500, R 30000-50000, 40 k x 6 z bins
    "echelle_sub": ("echelle_small", 12, (-1, -1), 0.0, None),
    "tiny_reso": ("tiny_reso", None, (-1, -1), 0.0, None),
    "tiny_reso_dia": ("tiny_reso_dia", None, (-1, -1), 0.0, None),
    # lyspeq's FastBootstrap (200 realizations) after the iteration of tiny_marg1
    "tiny_boot": ("tiny", None, (1, -1), 0.0, None, 200),
    # the complete bootstrap (FastBootstrap 0: a Fisher solve per realization)
    "tiny_boot_complete": ("tiny", None, (1, -1), 0.0, None, 100),
    # lyspeq's full Newton-Raphson loop (NumberOfIterations 4, smoothing between)
    "tiny_iter": ("tiny", None, (1, -1), 0.0, None, 0, 4),
    # noise-weight smoothing (Gaussian, and the mean) and redshift growth
    "tiny_smooth": ("tiny", None, (1, -1), 0.04, None),
    "tiny_smooth_mean": ("tiny", None, (-1, -1), 0.0, None),
    "tiny_reso_growth": ("tiny_reso", None, (-1, -1), 0.0, None),
    # SmoothResolutionMatrix (the matrices' diagonals smoothed before
    # deconvolution) with SmoothNoiseWeights 2
    "tiny_reso_smooth": ("tiny_reso", None, (-1, -1), 0.0, None),
    # top-hat redshift bins (RedshiftBinningMethod 0, bins::zBinTopHat)
    "tiny_tophat": ("tiny", None, (1, -1), 0.0, None),
    # TurnOffBaseline: C without the fiducial signal, no t trace
    "tiny_nosfid": ("tiny", None, (1, -1), 0.0, None),
    # DESI-size chunks with resolution matrices (11 diagonals deconvolved and
    # oversampled x3, N 160-634): the resolution path at the sizes it runs at
    "desi_reso_sub": ("desi_reso", 6, (-1, -1), 0.0, None),
    # the reference built with --enable-fisher-optimization (-DFISHER_OPTIMIZATION):
    # only the Fisher bands |dj| <= 5 and |dj - Nk| <= 2 are computed
    "desi_fopt": ("desi", 6, (1, -1), 0.0, None),
}

# cases whose redshift bins are top hats instead of triangles
TOPHAT = {"tiny_tophat"}

# cases run by the reference built with FISHER_OPTIMIZATION
FOPT = {"desi_fopt"}

# config keys set for a case: SmoothNoiseWeights and RedshiftGrowthOn
# (the growth exponent is the fiducial FiducialRedshiftPower)
OPTIONS = {
    "tiny_smooth": {"SmoothNoiseWeights": 3},
    "tiny_smooth_mean": {"SmoothNoiseWeights": 0},
    "tiny_reso_growth": {"RedshiftGrowthOn": 1},
    "tiny_reso_smooth": {"SmoothNoiseWeights": 2, "SmoothResolutionMatrix": 1},
    "tiny_nosfid": {"TurnOffBaseline": 1},
}


def _mask(w, frac, seed):
    if frac <= 0:
        return
    rng = np.random.Generator(np.random.PCG64(seed))
    for s in w.spectra:
        n = len(s.wave)
        idx = rng.choice(np.arange(1, n - 1), size=max(1, int(frac * n)), replace=False)
        s.sigma = s.sigma.copy()
        s.sigma[idx] = 1e10      # ivar = 1/sigma^2 < 1e-15 -> masked by the reader


def make_case(name, spec):
    wl, nch, marg, mask, keep = spec[:5]
    boots = spec[5] if len(spec) > 5 else 0
    iters = spec[6] if len(spec) > 6 else 1
    w = synth.make_workload(wl, n_chunks=nch)
    w.cont_logl_order, w.cont_l_order = marg
    if name in TOPHAT:
        w.bins.triangular = False
    _mask(w, mask, 99)
    with tempfile.TemporaryDirectory() as tmp:
        cfg = synth.write_reference_inputs(w, tmp)
        if iters > 1:
            text = open(cfg).read().replace("NumberOfIterations 1", f"NumberOfIterations {iters}")
            open(cfg, "w").write(text)
        opts = OPTIONS.get(name, {})
        if opts:
            text = open(cfg).read()
            for key, val in opts.items():
                if f"\n{key} " in text:
                    text = "\n".join(f"{key} {val}" if ln.startswith(f"{key} ") else ln for ln in text.split("\n"))
                else:
                    text += f"{key} {val}\n"
            open(cfg, "w").write(text)
        dump = refdump.run_driver(cfg, os.path.join(tmp, "dump.bin"), reso=w.reso, boots=boots,
                                  iterate=iters > 1, boot_complete=name.endswith("_complete"),
                                  fisher_optimization=name in FOPT)
        it = refdump.read_iteration(os.path.join(tmp, "dump.bin.iter")) if iters > 1 else None
    chunks = dump.chunks
    if keep is not None:
        chunks = chunks[:keep]
    out = dict(
        bins=np.array([w.bins.k0, w.bins.nklin, w.bins.dklin, w.bins.nklog, w.bins.dklog,
                       w.bins.z0, w.bins.dz, w.bins.nz, float(w.bins.triangular)]),
        grid=np.array([w.nv, w.lenv, w.nzp, w.max_forest_length, marg[0], marg[1]], dtype=float),
        table_r=np.array([t.r_fwhm for t in w.tables], dtype=np.int32),
        table_dv=np.array([t.dv for t in w.tables]),
        # tables are rebuilt from their definition by the tests; these sums detect drift
        table_sums=np.array([[np.abs(t.deriv).sum(), np.abs(t.signal).sum()] for t in w.tables]),
        n_chunks=np.array(len(chunks)),
        g_fisher=dump.fisher, g_dbt=dump.dbt, g_theta=dump.theta, g_solver=dump.solver_invfisher,
        g_inverse=dump.inverse_fisher, g_damped=np.array(dump.damped),
        g_complete=np.array(keep is None),
        # SmoothNoiseWeights, RedshiftGrowthOn, FiducialRedshiftPower,
        # SmoothResolutionMatrix, TurnOffBaseline
        opts=np.array([OPTIONS.get(name, {}).get("SmoothNoiseWeights", -1),
                       OPTIONS.get(name, {}).get("RedshiftGrowthOn", -1), w.fid[3],
                       OPTIONS.get(name, {}).get("SmoothResolutionMatrix", -1),
                       OPTIONS.get(name, {}).get("TurnOffBaseline", -1)], dtype=float),
    )
    if name in FOPT:
        out["fisher_opt"] = np.array(1)
    if it is not None:
        out["it_n"] = np.array(iters)
        out["it_theta"], out["it_prev"], out["it_fits"] = it.theta, it.previous, it.fits
        out["it_fisher"], out["it_inverse"], out["it_dbt"] = it.fisher, it.inverse, it.dbt
    if boots:
        out["boot_mean"] = dump.boot_mean
        out["boot_cov"] = dump.boot_cov
        out["boot_real"] = dump.boot_real
        out["boot_qso"] = np.array([c.qso for c in chunks], dtype=np.int32)
        out["boot_nqso"] = np.array(dump.n_qso)
        out["boot_complete"] = np.array([int(dump.boot_complete), dump.boot_valid])
    if w.reso:
        # resolution-matrix case: the reader's options, every spectrum's raw
        # matrix and wavelengths (for the preprocessing parity) and, per chunk,
        # the matrix as the reference's chunk holds it after deconvolution,
        # oversampling and the cuts
        out["reso"] = np.array([w.oversample, w.deconv_m])
        out["n_spectra"] = np.array(len(w.spectra))
        for j, sp in enumerate(w.spectra):
            out[f"s{j}_lam"] = sp.wave
            out[f"s{j}_resomat"] = sp.resomat
    for i, c in enumerate(chunks):
        # the chunk is a contiguous slice of its spectrum; keep the wavelengths in
        # Angstrom as read from the file so that lambda / LYA_REST is bit-identical
        full = w.spectra[c.qso].wave
        start = int(np.flatnonzero(full / LYA_REST == c.wave[0])[0])
        lam = full[start:start + c.n]
        assert np.array_equal(lam / LYA_REST, c.wave), "chunk is not a slice of its spectrum"
        out[f"c{i}_meta"] = np.array([c.n, c.fisher_index_start, c.nq, c.kbin_upp, c.r_fwhm,
                                      c.status], dtype=np.int64)
        out[f"c{i}_lam"] = lam
        out[f"c{i}_delta"] = c.delta
        out[f"c{i}_ivar"] = c.ivar
        out[f"c{i}_dbt"] = np.stack([c.d, c.b, c.t])
        out[f"c{i}_fisher"] = c.fisher
        if w.reso:
            out[f"c{i}_rmat"] = c.rmat
            out[f"c{i}_src"] = np.array([c.qso, start], dtype=np.int64)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {len(chunks)} chunks -> {os.path.getsize(path) / 1024:.0f} KiB")


def make_lyspeq_test():
    """lyspeq's own end-to-end test, as fixture lyspeq_test_it1: the binary
    spectrum file of tests/input (bytes), the numbers of tests/input/test.config
    and slist.txt the path needs, and the truth files of its first iteration
    (tests/truth/test_it1_fisher_matrix.dat, halved Fisher matrix, and the
    columns Pfid, ThetaP, Pest, ErrorP, the Fisher-weighted d, b, t and the
    d, b, t sums of test_it1_quadratic_power_estimate_detailed.dat)."""
    from oracle.refsrc import reference_root
    ref = reference_root()
    cfg = {}
    for line in open(os.path.join(ref, "tests", "input", "test.config")):
        parts = line.split()
        if len(parts) >= 2 and not parts[0].startswith("#"):
            cfg[parts[0]] = parts[1]
    fl = [ln.strip() for ln in open(os.path.join(ref, "tests", "input", "flist.txt")) if ln.strip()]
    sl = [ln.split() for ln in open(os.path.join(ref, "tests", "input", "slist.txt")) if ln.strip()]
    dat = np.frombuffer(open(os.path.join(ref, "tests", "input", fl[1]), "rb").read(), dtype=np.uint8)
    f = lambda k: float(cfg[k])
    bins = np.array([f("K0"), f("NumberOfLinearBins"), f("LinearKBinWidth"), f("NumberOfLog10Bins"),
                     f("Log10KBinWidth"), f("FirstRedshiftBinCenter"), f("RedshiftBinWidth"),
                     f("NumberOfRedshiftBins")])
    grid = np.array([f("NumberVPoints"), f("VelocityLength"), f("NumberZPoints"), f("MaximumForestLength"),
                     f("ContinuumLogLambdaMargOrder"), f("ContinuumLambdaMargOrder")])
    fid = np.array([f("FiducialAmplitude"), f("FiducialSlope"), f("FiducialCurvature"), f("FiducialRedshiftPower"),
                    f("FiducialRedshiftCurvature"), f("FiducialLorentzianLambda")])
    tables = np.array([[float(a), float(b)] for a, b in sl[1:]])
    truth = os.path.join(ref, "tests", "truth")
    with open(os.path.join(truth, "test_it1_quadratic_power_estimate_detailed.dat")) as fh:
        rows = [ln for ln in fh if not ln.startswith("#")]
    detailed = np.loadtxt(rows, skiprows=1)
    fisher = np.loadtxt(os.path.join(truth, "test_it1_fisher_matrix.dat"), skiprows=1)
    path = os.path.join(HERE, "lyspeq_test_it1.npz")
    np.savez_compressed(path, dat=dat, bins=bins, grid=grid, fid=fid, tables=tables,
                        detailed=detailed[:, 4:], fisher_halved=fisher)
    print(f"lyspeq_test_it1: {dat.size} bytes of spectrum -> {os.path.getsize(path) / 1024:.0f} KiB")


def main():
    if not refdump.available():
        raise SystemExit("oracle not built: make -C oracle/refbuild")
    names = sys.argv[1:] or list(CASES) + ["lyspeq_test_it1"]
    for name in names:
        if name == "lyspeq_test_it1":
            make_lyspeq_test()
        else:
            make_case(name, CASES[name])


if __name__ == "__main__":
    main()
