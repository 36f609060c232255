"""lqg_factor_noalloc: the allocation-free factorisation entry point.

Some callers cannot let a library allocate device memory inside their loop:
cudaMalloc and cudaFree may synchronise the whole device, which a host thread
with a latency budget cannot afford, and a caller that owns a fixed memory
pool must not have a library allocate behind its back.  This entry point takes
every buffer from the caller and keeps its only scratch in a fixed static
device array.

Checked on the GPU, through the C ABI, on two calls in a row:
* C^-1 and y against the oracle's inverse_covariance (the CPU restatement of
  Chunk::setInvertCovarianceMatrix and _addMarginalizations), to the FP64 bar;
* d, b, t and F recomputed on the host from them against the engine's own entry
  point (lqg_nr_iteration + lqg_chunk_result) on the same chunk;
* the same call in the self-checking build (-DLQG_CHECKED), whose index checks
  must accept the caller's buffers, which lie outside the static scratch.
This file runs last, so the calls also run after every other test has used the
device; each test also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import golden_cases as G

TOL = 1e-10


def _declare(lib):
    vp = C.c_void_p
    lib.lqg_factor_noalloc.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, C.c_int, C.c_int, vp, vp, vp]
    lib.lqg_factor_noalloc.restype = C.c_int
    return lib


def _lib():
    from lyspeq_gb300 import lqg
    return _declare(lqg.load_library())


def test_sizes_beyond_the_limit_are_rejected_before_any_device_work():
    lib = _lib()
    fake = C.c_void_p(16)   # never dereferenced: the size checks come first
    assert lib.lqg_factor_noalloc(5000, 5056, fake, fake, fake, fake, -1, -1, fake, fake, None) == -8
    assert lib.lqg_factor_noalloc(100, 100, fake, fake, fake, fake, -1, -1, fake, fake, None) == -1
    assert lib.lqg_factor_noalloc(100, 128, None, fake, fake, fake, -1, -1, fake, fake, None) == -1
    assert lib.lqg_factor_noalloc(100, 128, fake, fake, fake, fake, 3, 2, fake, fake, None) == -6


def _chunk():
    """The largest chunk of the tiny workload with amplitude + slope templates,
    its matrices and the oracle's C^-1 and y."""
    from lyspeq_gb300 import synth
    from oracle import qmle_port as P
    w = synth.make_workload("tiny")
    s = P.Settings(max_forest_length=w.max_forest_length, cont_logl_order=1, cont_l_order=-1)
    chunks = P.chunks_from_spectra(w.spectra, w.bins, w.table_index(), s)
    ch = max(chunks, key=lambda c: c.n)
    tv = P.table_view(w.tables[ch.res_index], w.bins, w.nv, w.lenv, w.nzp)
    stored, q, sm = P.build_matrices(ch, w.bins, tv)
    cinv = P.inverse_covariance(ch, stored, q, sm, np.zeros(w.bins.nkz), s)
    y = P._sym_upper(cinv) @ ch.delta
    return w, ch, stored, q, sm, cinv, y


def _run_twice(lib, ch, sm):
    """Two calls in a row on fresh device buffers; returns [(C^-1, y)] x 2."""
    import torch
    n = ch.n
    ld = (n + 63) // 64 * 64
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    wave = torch.tensor(ch.wave, dtype=torch.float64, device=dev)
    delta = torch.tensor(ch.delta, dtype=torch.float64, device=dev)
    ivar = torch.tensor(ch.ivar, dtype=torch.float64, device=dev)
    results = []
    for _ in range(2):
        cov = torch.zeros((ld, ld), dtype=torch.float64, device=dev)
        cov[:n, :n] = torch.tensor(sm, dtype=torch.float64, device=dev)
        y = torch.full((ld,), np.nan, dtype=torch.float64, device=dev)
        status = torch.full((1,), -99, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        rc = lib.lqg_factor_noalloc(n, ld, cov.data_ptr(), wave.data_ptr(), delta.data_ptr(),
                                    ivar.data_ptr(), 1, -1, y.data_ptr(), status.data_ptr(),
                                    C.c_void_p(stream.cuda_stream))
        assert rc == 0
        stream.synchronize()
        assert int(status.item()) == 0
        cinv = cov.cpu().numpy()
        assert np.all(cinv[n:, :] == 0) and np.all(cinv[:, n:] == 0)
        results.append((cinv[:n, :n].copy(), y.cpu().numpy()[:n].copy()))
    return results


@pytest.mark.gpu
def test_noalloc_factorisation_matches_the_oracle_and_the_engine_twice_in_a_row(engine_lib):
    from lyspeq_gb300 import lqg
    from oracle import qmle_port as P

    lib = _lib()
    w, ch, stored, q, sm, cinv_ref, y_ref = _chunk()

    # the existing entry point on the same chunk
    eng = lqg.Engine(w.bins, w.tables, w.nv, w.lenv, w.nzp, w.max_forest_length, cont=(1, -1))
    st = eng.add_chunk_list([(ch.wave * P.LYA_REST, ch.delta, ch.ivar, ch.r_fwhm)])
    assert (st == 0).all()
    eng.iterate(precision="fp64")
    ref = eng.chunk_result(0)
    eng.close()

    results = _run_twice(lib, ch, sm)
    n = ch.n
    for cinv, y in results:
        # C^-1 and y themselves, against the oracle
        assert G.rel_err(cinv, cinv_ref) < TOL
        assert G.rel_err(y, y_ref) < TOL
        # d, b, t, F of this chunk from C^-1 and y (core/chunk_estimate.cpp:746-834)
        nq = ch.nq
        d, b, t, f = np.zeros(nq), np.zeros(nq), np.zeros(nq), np.zeros((nq, nq))
        a = np.matmul(cinv[None], q)
        wn = np.zeros((n, n))
        good = ch.ivar != 0
        wn[good] = (1.0 / ch.ivar[good])[:, None] * cinv[good]
        ws = sm @ cinv
        for s_, ikz in enumerate(stored):
            d[ikz] = y @ (q[s_] @ y)
            b[ikz] = np.sum(a[s_] * wn)
            t[ikz] = np.sum(a[s_] * ws)
        idx = np.array(stored)
        full = np.einsum("ikl,jlk->ij", a, a)
        f[np.ix_(idx, idx)] = np.triu(full)
        assert G.rel_err(d, ref[0]) < TOL
        assert G.rel_err(b, ref[1]) < TOL
        assert G.rel_err(t, ref[2]) < TOL
        assert G.fisher_err(f, ref[3]) < TOL
    # the two calls are the same computation on the same inputs
    assert np.array_equal(results[0][0], results[1][0]) and np.array_equal(results[0][1], results[1][1])


@pytest.mark.gpu
def test_noalloc_runs_clean_in_the_self_checking_build(engine_lib):
    """The self-checking build skips and reports (status LQG_CHUNK_INDEX_CHECK)
    any index outside its buffers; the caller's C and y must pass its checks."""
    from lyspeq_gb300 import build
    lib = _declare(C.CDLL(build.build(checked=True)))
    _w, ch, _stored, _q, sm, cinv_ref, y_ref = _chunk()
    for cinv, y in _run_twice(lib, ch, sm):
        assert G.rel_err(cinv, cinv_ref) < TOL
        assert G.rel_err(y, y_ref) < TOL
