"""Resolution matrices (UseResoMatrix) through the C ABI.

* Host preprocessing (no GPU): lqg_resomat_deconvolve / lqg_resomat_oversample
  give the matrices lyspeq's own chunks hold (golden fixtures written by the
  reference compiled from its sources).
* GPU: the per-chunk results of the resolution-matrix cases are covered by the
  parametrised parity tests (test_gpu_parity.py at 1e-10, test_gpu_mixed.py at
  1e-5); here the NR step with nonzero theta, whose C = S + sum theta Q is
  formed per redshift bin on the resolution grid, is checked against the
  numpy restatement, and a batch mixing chunks with and without resolution
  matrices against the plain chunks alone.
"""
import numpy as np
import pytest

import golden_cases as G
from oracle import qmle_port as P


@pytest.mark.parametrize("name", G.RESO_CASES + G.RESO_SIZE_CASES)
def test_library_preprocessing_matches_reference(engine_lib, name):
    from lyspeq_gb300 import lqg
    c = G.load(name)
    osamp, m = c.reso
    prepared = {}
    for i, (qso, start) in enumerate(c.src):
        if qso not in prepared:
            lam, vals = c.spectra[qso]
            if c.smooth_rmat:
                vals = lqg.resomat_smooth(vals, c.opts["smooth_noise_weights"])
            v = lqg.resomat_deconvolve(vals, m) if m > 0 else np.array(vals)
            prepared[qso] = lqg.resomat_oversample(v, osamp, P._median(np.diff(lam))) if osamp > 0 else v
        n = c.meta[i][0]
        mine = prepared[qso][start:start + n] if osamp > 0 else prepared[qso][:, start:start + n]
        assert np.max(np.abs(mine - c.rmats[i])) < 1e-12


@pytest.mark.parametrize("sigmapix", [0, 1, 4])
def test_library_resomat_smoothing_matches_oracle(engine_lib, sigmapix):
    from lyspeq_gb300 import lqg
    rng = np.random.Generator(np.random.PCG64(8))
    vals = rng.uniform(0, 0.3, size=(11, 140))
    mine, ref = lqg.resomat_smooth(vals, sigmapix), P.smooth_rows(vals, sigmapix)
    assert np.max(np.abs(mine - ref)) <= 1e-15


def test_preprocessing_rejects_bad_arguments(engine_lib):
    from lyspeq_gb300 import lqg
    with pytest.raises(RuntimeError):
        lqg.resomat_deconvolve(np.ones((4, 10)), 1.0)       # even number of diagonals
    with pytest.raises(RuntimeError):
        lqg.resomat_oversample(np.ones((5, 10)), 0, 1.0)    # oversampling < 1


def _port_results(c, theta):
    s = c.port_settings(P)
    keys = {(t.r_fwhm, round(t.dv, 1)): i for i, t in enumerate(c.tables)}
    tv = P.table_view(c.tables[0], c.bins, c.nv, c.lenv, c.nzp)
    out = []
    for i, (lam, delta, ivar, r) in enumerate(c.chunks):
        ch = P.make_chunk(lam, delta, ivar, r, c.bins, keys, s, c.reso, c.rmats[i])
        out.append(P.chunk_iteration(ch, c.bins, tv, theta, s))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", G.RESO_CASES)
def test_nonzero_theta_matches_port(engine_lib, name):
    from test_gpu_parity import make_engine
    c = G.load(name)
    rng = np.random.Generator(np.random.PCG64(11))
    theta = 0.3 * c.g["theta"] + 0.01 * rng.standard_normal(c.bins.nkz)
    ref = _port_results(c, theta)
    eng, st = make_engine(c)
    assert (st == 0).all()
    eng.iterate(theta=theta, precision="fp64")
    for i, (d0, b0, t0, f0) in enumerate(ref):
        d, b, t, f = eng.chunk_result(i)
        assert G.rel_err(d, d0) < 1e-10 and G.rel_err(b, b0) < 1e-10 and G.rel_err(t, t0) < 1e-10
        assert G.fisher_err(f, f0) < 1e-10
    eng.iterate(theta=theta, precision="mixed")
    for i, (d0, b0, t0, f0) in enumerate(ref):
        d, b, t, f = eng.chunk_result(i)
        assert max(G.rel_err(d, d0), G.rel_err(b, b0), G.rel_err(t, t0), G.fisher_err(f, f0)) < 1e-5
    eng.close()


@pytest.mark.gpu
def test_batch_mixing_resolution_and_table_chunks(engine_lib):
    from lyspeq_gb300 import lqg
    cr = G.load("tiny_reso")
    cp = G.load("tiny_nomarg")
    # one context serving both kinds of chunk (the resolution chunks read table 0)
    eng = lqg.Engine(cp.bins, cp.tables, cp.nv, cp.lenv, cp.nzp, cp.max_forest_length, cont=cp.marg)
    st = eng.add_chunk_list(cp.chunks)
    assert (st == 0).all()
    eng.iterate(precision="fp64")
    alone = [eng.chunk_result(i) for i in range(eng.size)]
    st = eng.add_chunk_list_reso([ch[:3] + (rm,) for ch, rm in zip(cr.chunks, cr.rmats)], cr.reso[0])
    assert (st == 0).all()
    eng.iterate(precision="fp64")
    for i, (d0, b0, t0, f0) in enumerate(alone):
        d, b, t, f = eng.chunk_result(i)
        assert np.array_equal(d, d0) and np.array_equal(f, f0)
    eng.close()


@pytest.mark.gpu
def test_nonzero_theta_mixed_matches_fp64_on_desi_resolution_chunks(engine_lib):
    """The mixed path's theta term for resolution-matrix chunks comes from node
    tables of G(v) = sum_k theta_k Q_k(v) with cubic Hermite interpolation
    (error ~2e-8 of G) inside the double-float C build; the FP64 path sums the
    analytic band derivatives per grid element.  24 DESI-like resolution
    chunks at theta from a first NR step: every chunk's d, b, t and F within
    1e-5 of FP64, and the NR step itself (theta) within 1e-5 on the bins
    measured at 5 sigma or more."""
    from lyspeq_gb300 import lqg, synth
    w = synth.make_workload("desi_reso", n_chunks=24)
    eng = lqg.Engine(w.bins, w.tables, w.nv, w.lenv, w.nzp, w.max_forest_length,
                     cont=(w.cont_logl_order, w.cont_l_order))
    # each spectrum's matrix deconvolved and oversampled as lyspeq's reader does
    rr = []
    for s in w.spectra:
        v = lqg.resomat_deconvolve(s.resomat, w.deconv_m) if w.deconv_m > 0 else s.resomat
        rr.append(lqg.resomat_oversample(v, w.oversample, float(np.median(np.diff(s.wave))))
                  if w.oversample > 0 else v)
    st = eng.add_chunk_list_reso([(s.wave, s.delta, 1.0 / s.sigma ** 2, r) for s, r in zip(w.spectra, rr)],
                                 w.oversample)
    assert (st == 0).all()
    eng.iterate(precision="fp64")
    out = eng.download()
    theta = eng.fisher_solve(out["fisher"], np.stack([out["d"], out["b"], out["t"]]))["theta"]
    assert np.any(theta != 0)
    res = {}
    for prec in ("fp64", "mixed"):
        eng.iterate(theta=theta, precision=prec)
        o = eng.download()
        assert (o["status"] == 0).all()
        res[prec] = ([eng.chunk_result(i) for i in range(eng.size)],
                     eng.fisher_solve(o["fisher"], np.stack([o["d"], o["b"], o["t"]])))
    for (d, b, t, f), (d0, b0, t0, f0) in zip(res["mixed"][0], res["fp64"][0]):
        assert max(G.rel_err(d, d0), G.rel_err(b, b0), G.rel_err(t, t0), G.fisher_err(f, f0)) < 1e-5
    g0, g1 = res["fp64"][1], res["mixed"][1]
    sig = np.sqrt(np.abs(np.diag(g0["inverse"])))
    good = (sig > 0) & (np.abs(g0["theta"]) > 5 * sig)
    if good.any():
        assert np.max(np.abs(g1["theta"] - g0["theta"])[good] / np.abs(g0["theta"])[good]) < 1e-5
    eng.close()
