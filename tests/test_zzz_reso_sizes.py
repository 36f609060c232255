"""The resolution-matrix path at the sizes configuration 5 runs: six DESI-like
chunks of N 160-634 with 11-diagonal matrices deconvolved and oversampled x3
(fixture desi_reso_sub, from the compiled reference).  The FP64 path against
lyspeq's own results at 1e-10, the mixed path (the whitened form, which this
configuration runs) at 1e-5 per chunk and on the P1D of the global solution.  (The tiny_reso* fixtures of tests/test_gpu_parity.py
and tests/test_gpu_mixed.py hold a few short chunks.)
"""
import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu


def _engine(c):
    from lyspeq_gb300 import lqg
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg, **c.opts)
    st = eng.add_chunk_list_reso([ch[:3] + (rm,) for ch, rm in zip(c.chunks, c.rmats)], c.reso[0])
    assert (st == 0).all(), st
    return eng


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_desi_size_resolution_chunks_match_the_reference(engine_lib, precision, tol):
    c = G.load("desi_reso_sub")
    assert c.reso is not None and c.complete
    eng = _engine(c)
    for i, meta in enumerate(c.meta):
        info = eng.chunk_info(i)
        assert (info["n"], info["fisher_index_start"], info["nq"], info["kbin_upp"]) == meta[:4]
    eng.iterate(precision=precision)
    out = eng.download()
    assert (out["status"] == 0).all()
    for i, (dbt, fis) in enumerate(zip(c.dbt, c.fisher)):
        d, b, t, f = eng.chunk_result(i)
        errs = (G.rel_err(d, dbt[0]), G.rel_err(b, dbt[1]), G.rel_err(t, dbt[2]), G.fisher_err(f, fis))
        assert max(errs) < tol, (i, errs)
    g = eng.fisher_solve(out["fisher"], np.stack([out["d"], out["b"], out["t"]]))
    assert G.fisher_err(g["fisher"], c.g["fisher"]) < tol
    err, nbins = G.p1d_err(c.bins, c.g, g, c.g["fisher"])
    assert err < max(tol, 1e-9), (err, nbins)
    eng.close()
