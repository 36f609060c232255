"""The Poisson bootstraps against lyspeq's own PoissonBootstrapper run by the
compiled reference on the same chunks: FastBootstrap (lqg_bootstrap, golden
fixture tiny_boot: 200 realizations over 6 spectra) and the complete bootstrap
(lqg_bootstrap_complete, fixture tiny_boot_complete: 100 realizations, a
Cholesky solve each).  The Poisson coefficients come from the same generator,
so realizations, mean and covariance agree to rounding.

On the CPU: the oracle's restatement of the complete bootstrap, fed the
reference's own per-chunk results and the library's coefficients, reproduces
the fixture."""
import numpy as np
import pytest

import golden_cases as G
from oracle import qmle_port as P


def _offsets(c):
    return np.searchsorted(c.boot["qso"], np.arange(c.boot["n_qso"] + 1), side="left")


def test_complete_bootstrap_oracle_matches_reference(engine_lib):
    from lyspeq_gb300 import lqg
    c = G.load("tiny_boot_complete")
    assert c.boot["complete"]
    nb = c.boot["real"].shape[0]
    off = _offsets(c)
    p = lqg.bootstrap_coefficients(c.boot["n_qso"], nb, seed=0, per_realization=True)
    chunks = [(m[1], m[2], dbt[0], dbt[1], dbt[2], f) for m, dbt, f in zip(c.meta, c.dbt, c.fisher)]
    slots, nv, mean, cov = P.complete_bootstrap(c.bins.nkz, chunks, off, p)
    assert nv == c.boot["valid"]
    assert G.rel_err(slots, c.boot["real"]) < 1e-10
    assert G.rel_err(mean, c.boot["mean"]) < 1e-10
    assert G.rel_err(cov, c.boot["cov"]) < 1e-10


def test_bootstrap_coefficient_orders(engine_lib):
    """Both draw orders take the same stream: FastBootstrap nboots per
    spectrum, the complete bootstrap one per spectrum per realization."""
    from lyspeq_gb300 import lqg
    fast = lqg.bootstrap_coefficients(5, 7, seed=3)
    full = lqg.bootstrap_coefficients(5, 7, seed=3, per_realization=True)
    assert np.array_equal(fast.ravel(), full.T.ravel())
    assert 0.9 < fast.mean() < 1.1 or fast.size < 100


@pytest.mark.gpu
def test_complete_bootstrap_matches_reference(engine_lib):
    from lyspeq_gb300 import lqg
    c = G.load("tiny_boot_complete")
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg)
    assert (eng.add_chunk_list(c.chunks) == 0).all()
    eng.iterate(precision="fp64")
    nb = c.boot["real"].shape[0]
    out = eng.bootstrap_complete(_offsets(c), nb, seed=0)
    assert out["n_valid"] == c.boot["valid"]
    assert G.rel_err(out["realizations"], c.boot["real"]) < 1e-9
    assert G.rel_err(out["mean"], c.boot["mean"]) < 1e-9
    assert G.rel_err(out["cov"], c.boot["cov"]) < 1e-9
    eng.close()


@pytest.mark.gpu
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


@pytest.mark.gpu
def test_bootstrap_needs_an_iteration(engine_lib):
    from lyspeq_gb300 import lqg
    c = G.load("tiny_boot")
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg)
    eng.add_chunk_list(c.chunks)
    with pytest.raises(RuntimeError):
        eng.bootstrap([0, len(c.chunks)], 10)
    eng.close()
