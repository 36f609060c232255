"""The autotuner of the mixed path's launch plan (lqg_autotune, lqg_tuning_*).

Per padded chunk size it picks the form (whitened or direct), the products'
drain interval and the Gram's K split, keeping only plans whose per-chunk
results stay within the error bound of the FP64 path; LQG_PRECISION_MIXED_AUTO
iterations follow the table.
"""
import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu


def _desi(n=48):
    from lyspeq_gb300 import lqg, synth
    w = synth.make_workload("desi", n_chunks=n)
    eng = lqg.Engine(w.bins, w.tables, w.nv, w.lenv, w.nzp, w.max_forest_length, cont=(1, -1))
    st = eng.add_chunk_list([(s.wave, s.delta, 1.0 / s.sigma ** 2, s.r_fwhm) for s in w.spectra])
    assert (st == 0).all()
    return eng


def _results(eng):
    return [eng.chunk_result(i) for i in range(eng.size)]


def test_a_fixed_table_reproduces_the_fixed_modes_bit_for_bit(engine_lib):
    eng = _desi()
    lds = sorted({(eng.chunk_info(i)["n"] + 63) // 64 * 64 for i in range(eng.size)})
    for sym, mode in ((1, "mixed"), (0, "mixed_direct")):
        eng.iterate(precision=mode)
        ref = _results(eng)
        eng.set_tuning([(ld, sym, 8, 32768, 0) for ld in lds])
        t = eng.tuning()
        assert t.shape == (len(lds), 5) and (t[:, 1] == sym).all()
        eng.iterate(precision="mixed_auto")
        for x, y in zip(_results(eng), ref):
            for a, b in zip(x, y):
                assert np.array_equal(a, b)
    with pytest.raises(RuntimeError):
        eng.set_tuning([(100, 1, 8, 32768, 0)])   # ld must be a multiple of 64
    with pytest.raises(RuntimeError):
        eng.set_tuning([(lds[0], 1, 8, 32768, 2)])   # pair is 0 or 1
    eng.close()


def test_autotuned_plan_meets_the_bar_against_fp64(engine_lib):
    eng = _desi()
    table = eng.autotune(max_rel_err=1e-5, max_chunks=16)
    lds = sorted({(eng.chunk_info(i)["n"] + 63) // 64 * 64 for i in range(eng.size)})
    assert [int(r[0]) for r in table] == lds
    assert set(table[:, 1]) <= {0, 1} and set(table[:, 2]) <= {4, 8, 16} and set(table[:, 3]) <= {16384, 32768, 65536}
    assert set(table[:, 4]) <= {0, 1}
    eng.iterate(precision="fp64")
    ref = _results(eng)
    eng.iterate(precision="mixed_auto")
    out = eng.download()
    assert (out["status"] == 0).all()
    for (d, b, t, f), (rd, rb, rt, rf) in zip(_results(eng), ref):
        assert max(G.rel_err(d, rd), G.rel_err(b, rb), G.rel_err(t, rt), G.fisher_err(f, rf)) < 1e-5
    # the table survives a round trip (a caller persists it between runs)
    eng.set_tuning(table)
    assert np.array_equal(eng.tuning(), table)
    eng.close()


@pytest.mark.parametrize("sym", [1, 0])
def test_cta_pair_products_match_the_single_cta_kernel(engine_lib, sym):
    """k_tc_gemm_pair (256 x 128 tiles on two CTAs) against k_tc_gemm on every
    padded size of the sample, both forms: the same products but for the
    drain interval of the slot paired with S (whitened form), so close to
    each other (5e-6) and within the bar of FP64; every chunk's status ok."""
    eng = _desi()
    lds = sorted({(eng.chunk_info(i)["n"] + 63) // 64 * 64 for i in range(eng.size)})
    eng.iterate(precision="fp64")
    ref = _results(eng)
    out = []
    for pair in (0, 1):
        eng.set_tuning([(ld, sym, 8, 32768, pair) for ld in lds])
        eng.iterate(precision="mixed_auto")
        assert (eng.download()["status"] == 0).all()
        out.append(_results(eng))
    for single, paired, fp64 in zip(out[0], out[1], ref):
        assert max(G.rel_err(x, y) for x, y in zip(paired[:3], single[:3])) < 5e-6
        assert G.fisher_err(paired[3], single[3]) < 5e-6
        assert max(G.rel_err(x, y) for x, y in zip(paired[:3], fp64[:3])) < 1e-5
        assert G.fisher_err(paired[3], fp64[3]) < 1e-5
    eng.close()
