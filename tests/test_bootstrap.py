"""FastBootstrap (lqg_bootstrap) against lyspeq's own PoissonBootstrapper run
by the compiled reference on the same chunks (golden fixture tiny_boot: 200
realizations over 6 spectra).  The Poisson coefficients come from the same
generator, so realizations, mean and covariance agree to rounding (1e-12)."""
import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu


def test_fast_bootstrap_matches_reference(engine_lib):
    from lyspeq_gb300 import lqg
    c = G.load("tiny_boot")
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg)
    assert (eng.add_chunk_list(c.chunks) == 0).all()
    eng.iterate(precision="fp64")
    qso = c.boot["qso"]
    off = np.searchsorted(qso, np.arange(c.boot["n_qso"] + 1), side="left")
    nb = c.boot["real"].shape[0]
    out = eng.bootstrap(off, nb, seed=0, solver=c.g["solver"], realizations=True)
    assert G.rel_err(out["realizations"], c.boot["real"]) < 1e-12
    assert G.rel_err(out["mean"], c.boot["mean"]) < 1e-12
    assert G.rel_err(out["cov"], c.boot["cov"]) < 1e-11
    # mixed-precision chunks give the same bootstrap to the mixed path's bar
    eng.iterate(precision="mixed")
    out = eng.bootstrap(off, nb, seed=0, solver=c.g["solver"])
    assert G.rel_err(out["mean"], c.boot["mean"]) < 1e-5
    eng.close()


def test_bootstrap_needs_an_iteration(engine_lib):
    from lyspeq_gb300 import lqg
    c = G.load("tiny_boot")
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg)
    eng.add_chunk_list(c.chunks)
    with pytest.raises(RuntimeError):
        eng.bootstrap([0, len(c.chunks)], 10)
    eng.close()
