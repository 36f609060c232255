"""SQ lookup tables generated on the GPU (lqg_tables_generate) against the
table builder of lyspeq_gb300.synth, which reproduces lyspeq's own truth
table tests/truth/signal_R70000_dv20.0.fits to 1e-12 (tests/test_oracle.py).
Bar: max |difference| <= 1e-12 max |table| for the derivative and signal
tables."""
import numpy as np
import pytest

from lyspeq_gb300 import synth

pytestmark = pytest.mark.gpu


def _compare(bins, pairs, nv, lenv, nzp, fid=synth.PD13_DEFAULT):
    from lyspeq_gb300 import lqg
    deriv, signal = lqg.generate_tables(bins, pairs, nv, lenv, nzp, fid)
    for t, (r, dv) in enumerate(pairs):
        ref = synth.build_table(bins, r, dv, nv, lenv, nzp, fid=fid)
        assert np.max(np.abs(deriv[t] - ref.deriv)) <= 1e-12 * np.max(np.abs(ref.deriv))
        assert np.max(np.abs(signal[t] - ref.signal)) <= 1e-12 * np.max(np.abs(ref.signal))


def test_truth_table_configuration(engine_lib):
    # the binning, grids and fiducial of lyspeq's truth table (R 70000, dv 20)
    bins = synth.Bins(0.0, 3, 7e-4, 2, 0.5, 1.8, 0.2, 2)
    _compare(bins, [(70000, 20.0)], 1401, 14000.0, 10, fid=(0.06, -2.6, -0.1, 1.0, 0.0, 0.0))


def test_desi_like_tables(engine_lib):
    w = synth.make_workload("desi", n_chunks=8)
    pairs = [(t.r_fwhm, t.dv) for t in w.tables[:3]]
    _compare(w.bins, pairs, w.nv, w.lenv, w.nzp)


def test_echelle_like_tables(engine_lib):
    # many (R, dv) pairs with small dv: long velocity grids, 40 k bands
    w = synth.make_workload("echelle", n_chunks=3)
    pairs = [(t.r_fwhm, t.dv) for t in w.tables]
    _compare(w.bins, pairs, w.nv, w.lenv, w.nzp)


def test_generated_tables_drive_the_engine(engine_lib):
    import golden_cases as G
    from lyspeq_gb300 import lqg
    c = G.load("tiny_marg1")
    pairs = [(t.r_fwhm, t.dv) for t in c.tables]
    deriv, signal = lqg.generate_tables(c.bins, pairs, c.nv, c.lenv, c.nzp, synth.PD13_DEFAULT)
    tabs = [synth.Table(t.r_fwhm, t.dv, c.nv, c.lenv, c.nzp, t.z1, t.lenz, deriv[i], signal[i])
            for i, t in enumerate(c.tables)]
    eng = lqg.Engine(c.bins, tabs, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg)
    assert (eng.add_chunk_list(c.chunks) == 0).all()
    eng.iterate(precision="fp64")
    for i, (dbt, fis) in enumerate(zip(c.dbt, c.fisher)):
        d, b, t, f = eng.chunk_result(i)
        assert G.rel_err(d, dbt[0]) < 1e-9 and G.fisher_err(f, fis) < 1e-9
    eng.close()
