"""Failure paths of the engine, exercised without faulting the GPU.

* Bounded waits: every wait inside the tensor-core kernels has a wall-clock
  limit (lqg_set_wait_limit).  With a 1 ns limit the first wait that is not
  already satisfied runs out; its CTA stops issuing, drains its own copies and
  MMAs (those waits keep 2 s), frees its tensor memory and marks its chunks
  LQG_CHUNK_TIMEOUT.  The call returns, those chunks contribute nothing (as
  the reference skips a chunk that throws, core/chunk_estimate.cpp:905-913),
  and the next iteration on the same context is exact again.
  The same on CTA pairs (k_tc_gemm_pair), where a wait that runs out in one
  CTA also stops the other.
* The self-checking build (-DLQG_CHECKED): every device index is checked
  against its buffer, a violation is counted and the access skipped.  The
  golden cases run through it with no violation and the usual parity, the
  products on one CTA and on CTA pairs.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TIMEOUT = 8   # LQG_CHUNK_TIMEOUT


def _engine(c):
    from lyspeq_gb300 import lqg
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg, **c.opts)
    assert (eng.add_chunk_list(c.chunks) == 0).all()
    return eng


def _plan(eng, mode):
    """The precision to iterate with: the fixed modes, or the products on CTA
    pairs (whitened or direct form) through a tuning table."""
    if not mode.startswith("pair"):
        return mode
    lds = sorted({(eng.chunk_info(i)["n"] + 63) // 64 * 64 for i in range(eng.size)})
    eng.set_tuning([(ld, 1 if mode == "pair_whitened" else 0, 8, 32768, 1) for ld in lds])
    return "mixed_auto"


@pytest.mark.parametrize("mode", ["mixed", "mixed_direct", "pair_whitened", "pair_direct"])
def test_waits_that_run_out_drop_their_chunks_and_the_next_iteration_is_exact(engine_lib, mode):
    c = G.load("tiny_marg1")
    eng = _engine(c)
    precision = _plan(eng, mode)
    eng.set_wait_limit(1e-9)
    eng.iterate(precision=precision)
    out = eng.download()
    st = out["status"]
    assert (st == TIMEOUT).any(), st
    assert set(np.unique(st).tolist()) <= {0, TIMEOUT}
    # timed-out chunks contribute nothing: the sums are those of the others
    keep = np.flatnonzero(st == 0)
    dsum = np.zeros(c.bins.nkz)
    for i in keep:
        m = c.meta[i]
        dsum[m[1]:m[1] + m[2]] += eng.chunk_result(int(i))[0]
    np.testing.assert_allclose(out["d"], dsum, rtol=1e-12, atol=0)
    for i in np.flatnonzero(st == TIMEOUT):
        d, b, t, f = eng.chunk_result(int(i))
        assert not d.any() and not b.any() and not t.any() and not f.any()

    eng.set_wait_limit(0)
    eng.iterate(precision=precision)
    out = eng.download()
    assert (out["status"] == 0).all()
    for i, (dbt, fis) in enumerate(zip(c.dbt, c.fisher)):
        d, b, t, f = eng.chunk_result(i)
        assert max(G.rel_err(d, dbt[0]), G.rel_err(b, dbt[1]), G.rel_err(t, dbt[2]),
                   G.fisher_err(f, fis)) < 1e-5
    eng.close()


CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, "tests")
import golden_cases as G
from lyspeq_gb300 import lqg
for name in ["tiny_marg1", "tiny_masked", "tiny_marg3", "tiny_nosfid", "tiny_reso", "tiny_reso_dia", "desi_sub"]:
    c = G.load(name)
    # tiny_marg3's templates are nearly collinear: the reference itself is
    # determined to ~1e-8 there, and the mixed forms are not held to 1e-5 on it
    # (tests/test_gpu_parity.py, tests/test_gpu_mixed.py)
    runs = (("fp64", 1e-7),) if name == "tiny_marg3" else (("fp64", 1e-9), ("mixed", 1e-5), ("mixed_direct", 1e-5),
                                                            ("pair", 1e-5))
    for precision, tol in runs:
        eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg, **c.opts)
        if c.reso is None:
            st = eng.add_chunk_list(c.chunks)
        else:
            st = eng.add_chunk_list_reso([ch[:3] + (rm,) for ch, rm in zip(c.chunks, c.rmats)], c.reso[0])
        assert (st == 0).all(), (name, st)
        if precision == "pair":
            # the products on CTA pairs (k_tc_gemm_pair), whitened form
            lds = sorted({(eng.chunk_info(i)["n"] + 63) // 64 * 64 for i in range(eng.size)})
            eng.set_tuning([(ld, 1, 8, 32768, 1) for ld in lds])
            precision = "mixed_auto"
        for _ in range(2):   # the second iteration replays a captured graph
            eng.iterate(precision=precision)   # raises if an index check failed
            out = eng.download()
            assert (out["status"] == 0).all(), (name, precision, out["status"])
            for i, (dbt, fis) in enumerate(zip(c.dbt, c.fisher)):
                d, b, t, f = eng.chunk_result(i)
                err = max(G.rel_err(d, dbt[0]), G.rel_err(b, dbt[1]), G.rel_err(t, dbt[2]), G.fisher_err(f, fis))
                assert err < tol, (name, precision, i, err)
        eng.close()
print("checked build clean")
"""


def test_golden_cases_run_clean_in_the_self_checking_build(engine_lib):
    from lyspeq_gb300 import build
    lib = build.build(checked=True)
    env = dict(os.environ, LQG_LIB=lib)
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "checked build clean" in r.stdout
