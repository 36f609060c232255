"""lyspeq built with FISHER_OPTIMIZATION (lqg_set_fisher_optimization).

The reference built with ./configure --enable-fisher-optimization computes of
each chunk's Fisher matrix only the pairs of local kz indices i <= j with
j - i <= 5 or |j - i - Nk| <= 2 (core/chunk_estimate.cpp:823-827) and leaves
the rest 0.  The fixture desi_fopt holds its results on the six DESI-like
chunks of desi_sub (Nk = 35).  The engine with the option on must give the
same zeros, the kept elements and d, b, t at the bars of each path, and the
global solution of the banded sum; with the option off again, the full
matrices of desi_sub.
"""
import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu


def _engine(c):
    from lyspeq_gb300 import lqg
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg, **c.opts)
    assert (eng.add_chunk_list(c.chunks) == 0).all()
    return eng


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_banded_fisher_matrices_match_the_reference(engine_lib, precision, tol):
    from lyspeq_gb300 import lqg
    c = G.load("desi_fopt")
    assert c.fisher_optimization
    eng = _engine(c)
    eng.set_fisher_optimization(True)
    eng.iterate(precision=precision)
    out = eng.download()
    assert (out["status"] == 0).all()
    for i, (dbt, fis) in enumerate(zip(c.dbt, c.fisher)):
        d, b, t, f = eng.chunk_result(i)
        assert np.array_equal(f == 0, fis == 0), i
        assert G.fisher_err(f, fis) < tol, (i, G.fisher_err(f, fis))
        scale = max(np.max(np.abs(dbt[1])), np.max(np.abs(dbt[2])))
        assert G.rel_err(d, dbt[0]) < tol, i
        assert np.max(np.abs(b - dbt[1])) < tol * scale and np.max(np.abs(t - dbt[2])) < tol * scale, i
    # the global sum is the banded one: its solution against the reference's
    fsum, dbt = G.global_sums(c)
    g = eng.fisher_solve(out["fisher"], np.stack([out["d"], out["b"], out["t"]]))
    assert G.fisher_err(g["fisher"], c.g["fisher"]) < tol
    g_ref = lqg.fisher_solve(fsum, dbt)
    assert G.rel_err(g_ref["theta"], c.g["theta"]) < 1e-9
    err, nbins = G.p1d_err(c.bins, g_ref, g, fsum)
    # the banded global matrix of these chunks is indefinite (two negative
    # eigenvalues, condition 1.6e8), which amplifies the mixed path's per-element
    # errors (bounded above at 1e-5) into P1D: 2.1e-5 measured on its two bins
    # at 5 sigma; the FP64 path keeps its 1e-10
    p1d_tol = 1e-9 if precision == "fp64" else 5e-5
    assert nbins > 0 and err < p1d_tol, (err, nbins)
    # off again: the full matrices of the same chunks
    eng.set_fisher_optimization(False)
    eng.iterate(precision=precision)
    full = G.load("desi_sub")
    for i, fis in enumerate(full.fisher):
        assert G.fisher_err(eng.chunk_result(i)[3], fis) < tol, i
    assert eng.lib.lqg_set_fisher_optimization(eng.h, 2) == -1   # LQG_ERR_ARG
    eng.close()
