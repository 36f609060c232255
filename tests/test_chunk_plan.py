"""Chunk::Chunk on the host without a GPU (lqg_chunk_plan): the same code that
lqg_batch_add runs, checked against the oracle's make_chunk (pinned to the
compiled reference's chunks in tests/test_oracle.py).

Cases: every golden table case (their chunks as lyspeq built them), the small
workload's raw spectra as chunks (many outside the redshift bins, where the
engine's guard says LQG_CHUNK_OUT_OF_RANGE; the reference's reader would
have cut them), and planted faults: masked ends, everything masked, too few
pixels, sparse pixels, an unknown resolution, a non-finite value.
"""
import numpy as np
import pytest

import golden_cases as G
from oracle import qmle_port as P

OK, SHORT, NO_TABLE, EMPTY, OUT_OF_RANGE, BAD_INPUT = 0, 1, 2, 3, 4, 6


def _plan(bins, tables, chunks, mfl):
    from lyspeq_gb300 import lqg
    offs = np.cumsum([0] + [len(c[0]) for c in chunks])
    cat = lambda j: np.concatenate([np.asarray(c[j], dtype=np.float64) for c in chunks])
    return lqg.chunk_plan(bins, tables, cat(0), cat(1), cat(2), offs, [c[3] for c in chunks], mfl)


def _compare(bins, tables, chunks, mfl):
    """Every chunk accepted by both with the same numbers, or rejected by
    both; returns the statuses."""
    keys = {(t.r_fwhm, round(t.dv, 1)): i for i, t in enumerate(tables)}
    s = P.Settings(max_forest_length=mfl)
    status, info = _plan(bins, tables, chunks, mfl)
    for (lam, d, iv, r), code, inf in zip(chunks, status, info):
        try:
            ch = P.make_chunk(np.asarray(lam), np.asarray(d), np.asarray(iv), r, bins, keys, s)
        except (ValueError, KeyError):
            assert code in (SHORT, NO_TABLE, EMPTY), code
            continue
        except IndexError:
            # beyond the last redshift bin, where the restatement (like the
            # reference, whose reader cuts spectra first) has no bin to index
            assert code == OUT_OF_RANGE
            continue
        if ch.zbin_low < 0 or ch.zbin_upp >= bins.nz:
            assert code == OUT_OF_RANGE
            continue
        assert code == OK
        assert (inf["n"], inf["fisher_index_start"], inf["nq"], inf["kbin_upp"], inf["res_index"],
                inf["zbin_low"], inf["zbin_upp"]) == (ch.n, ch.fisher_index_start, ch.nq, ch.kbin_upp,
                                                      ch.res_index, ch.zbin_low, ch.zbin_upp)
    return status


@pytest.mark.parametrize("name", [n for n in G.CASES if n not in G.RESO_CASES])
def test_golden_chunks(engine_lib, name):
    c = G.load(name)
    status = _compare(c.bins, c.tables, c.chunks, c.max_forest_length)
    assert (status == OK).all()
    _, info = _plan(c.bins, c.tables, c.chunks, c.max_forest_length)
    assert [(i["n"], i["fisher_index_start"], i["nq"], i["kbin_upp"]) for i in info] == [m[:4] for m in c.meta]


def test_raw_spectra_and_planted_faults(engine_lib):
    from lyspeq_gb300 import synth
    w = synth.make_workload("small")
    raw = [(s.wave, s.delta, 1.0 / np.asarray(s.sigma) ** 2, s.r_fwhm) for s in w.spectra]
    status = _compare(w.bins, w.tables, raw, w.max_forest_length)
    assert (status == OK).sum() > 0 and (status == OUT_OF_RANGE).sum() > 0
    # planted faults on an accepted chunk
    base = next(c for c, st in zip(raw, status) if st == OK)
    lam, d, iv, r = (np.array(x) if i < 3 else x for i, x in enumerate(base))
    iv_ends = iv.copy()
    iv_ends[:7] = 0
    iv_ends[-3:] = 0
    # keep one pixel in `stride`: a mean pixel size above MaximumMeanPixelSize
    dv = 299792.458 * np.log(lam[1] / lam[0])
    stride = int(np.ceil(150.0 / dv)) + 1
    iv_sparse = np.where(np.arange(len(iv)) % stride == 0, iv, 0.0)
    d_nan = d.copy()
    d_nan[5] = np.nan
    planted = [(lam, d, iv_ends, r), (lam, d, np.zeros_like(iv), r), (lam[:3], d[:3], iv[:3], r),
               (lam, d, iv_sparse, r), (lam, d, iv, r + 1), (lam, d_nan, iv, r)]
    status, info = _plan(w.bins, w.tables, planted, w.max_forest_length)
    assert list(status) == [OK, EMPTY, SHORT, SHORT, NO_TABLE, BAD_INPUT]
    assert info[0]["n"] == len(lam) - 10        # the masked ends are cut
    _compare(w.bins, w.tables, planted[:5], w.max_forest_length)


@pytest.mark.parametrize("name", G.RESO_CASES + G.RESO_SIZE_CASES)
def test_resolution_matrix_chunks(engine_lib, name):
    """Chunks with resolution matrices (lqg_batch_add_reso's rules: RES_INDEX 0,
    no table lookup), per-pixel rows as add_chunk_list_reso passes them."""
    from lyspeq_gb300 import lqg
    c = G.load(name)
    osamp = c.reso[0]
    rows = [np.asarray(rm) if osamp > 0 else np.asarray(rm).T for rm in c.rmats]
    offs = np.cumsum([0] + [len(x[0]) for x in c.chunks])
    cat = lambda j: np.concatenate([np.asarray(x[j], dtype=np.float64) for x in c.chunks])
    status, info = lqg.chunk_plan(c.bins, c.tables, cat(0), cat(1), cat(2), offs, None, c.max_forest_length,
                                  oversampling=osamp, resomat=np.concatenate(rows))
    assert (status == OK).all()
    keys = {(t.r_fwhm, round(t.dv, 1)): i for i, t in enumerate(c.tables)}
    s = c.port_settings(P)
    for (lam, d, iv, r), rm, m, inf in zip(c.chunks, c.rmats, c.meta, info):
        ch = P.make_chunk(np.asarray(lam), np.asarray(d), np.asarray(iv), r, c.bins, keys, s, c.reso, rm)
        got = (inf["n"], inf["fisher_index_start"], inf["nq"], inf["kbin_upp"], inf["res_index"])
        assert got == (ch.n, ch.fisher_index_start, ch.nq, ch.kbin_upp, ch.res_index) == tuple(m[:4]) + (0,)
