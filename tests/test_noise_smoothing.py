"""Noise-weight smoothing (SmoothNoiseWeights) and redshift growth (RedshiftGrowthOn).

* The library's host smoother (lqg_smooth_ivar) against the oracle's
  restatement of Smoother::smoothIvar, which the golden fixtures tiny_smooth
  and tiny_smooth_mean pin to lyspeq's own outputs (tests/test_oracle.py).
* Both options through the engine: the GPU parity tests run the fixtures
  tiny_smooth, tiny_smooth_mean and tiny_reso_growth like every other case
  (tests/test_gpu_parity.py, tests/test_gpu_mixed.py); here the plain-table
  growth path, which has no reference fixture, is checked against the oracle.
"""
import numpy as np
import pytest

import golden_cases as G
from oracle import qmle_port as P


def _ivars():
    rng = np.random.Generator(np.random.PCG64(21))
    out = []
    for n, first, last in ((160, False, False), (300, True, False), (120, False, True), (60, True, True),
                           (30, False, False)):
        iv = 1.0 / rng.lognormal(np.log(0.2), 0.6, size=n) ** 2
        iv[rng.choice(n, size=max(1, n // 20), replace=False)] = 0.0
        iv[0] = 0.0 if first else iv[0]
        iv[-1] = 1e-9 if last else iv[-1]      # far below the high-noise cut
        out.append(iv)
    return out


@pytest.mark.parametrize("sigmapix", [0, 1, 3, 7])
def test_library_smoothing_matches_oracle(engine_lib, sigmapix):
    from lyspeq_gb300 import lqg
    for iv in _ivars():
        mine, ref = lqg.smooth_ivar(iv, sigmapix), P.smooth_ivar(iv, sigmapix)
        assert np.array_equal(mine == 0, ref == 0)
        assert np.max(np.abs(mine - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_smoothing_keeps_the_reference_padding(engine_lib):
    """padArray's right-hand pad lands on the last 25 pixels and leaves zeros
    past them: those pixels get ivar 0 unless the last pixel is masked (then
    the fill replaces the zeros and the last pixel keeps its own ivar)."""
    from lyspeq_gb300 import lqg
    iv = np.full(200, 4.0)
    out = lqg.smooth_ivar(iv, 3)
    assert np.all(out[-25:] == 0) and np.allclose(out[:-25], 4.0, rtol=1e-14)
    iv[-1] = 1e-9                      # a high-noise last pixel counts as masked
    out = lqg.smooth_ivar(iv, 3)
    assert out[-1] == 1e-9 and np.all(out > 0)
    assert np.allclose(out[:-50], 4.0, rtol=1e-14)


def test_smoothing_rejects_bad_arguments(engine_lib):
    from lyspeq_gb300 import lqg
    with pytest.raises(RuntimeError):
        lqg.smooth_ivar(np.ones(10), -1)
    with pytest.raises(RuntimeError):
        lqg.smooth_ivar(np.ones(0), 3)


@pytest.mark.gpu
def test_growth_on_table_chunks_matches_oracle(engine_lib):
    """RedshiftGrowthOn without a resolution matrix: the engine scales Q_k by
    ((1 + z_ij) / (1 + z_m))^B on the symmetric z_ij, as the oracle does."""
    from lyspeq_gb300 import lqg
    c = G.load("tiny_marg1")
    opts = dict(smooth_noise_weights=3, redshift_growth=True, fid_b=3.591244)
    s = P.Settings(max_forest_length=c.max_forest_length, cont_logl_order=c.marg[0], cont_l_order=c.marg[1],
                   smooth_noise_weights=3, redshift_growth=True, growth_b=3.591244)
    keys = {(t.r_fwhm, round(t.dv, 1)): i for i, t in enumerate(c.tables)}
    tvs = [P.table_view(t, c.bins, c.nv, c.lenv, c.nzp) for t in c.tables]
    rng = np.random.Generator(np.random.PCG64(3))
    theta = 0.3 * c.g["theta"] + 0.01 * rng.standard_normal(c.bins.nkz)
    ref = []
    for lam, delta, ivar, r in c.chunks:
        ch = P.make_chunk(lam, delta, ivar, r, c.bins, keys, s)
        ref.append(P.chunk_iteration(ch, c.bins, tvs[ch.res_index], theta, s))
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg, **opts)
    assert (eng.add_chunk_list(c.chunks) == 0).all()
    for precision, tol in (("fp64", 1e-10), ("mixed", 1e-5)):
        eng.iterate(theta=theta, precision=precision)
        for i, (d0, b0, t0, f0) in enumerate(ref):
            d, b, t, f = eng.chunk_result(i)
            errs = (G.rel_err(d, d0), G.rel_err(b, b0), G.rel_err(t, t0), G.fisher_err(f, f0))
            assert max(errs) < tol, (precision, i, errs)
    eng.close()
