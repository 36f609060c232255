"""Newton-Raphson loop with smoothing (lyspeq_gb300.estimator) against
lyspeq's own OneDQuadraticPowerEstimate::iterate run by the compiled
reference (golden fixture tiny_iter: NumberOfIterations 4, the estimate
smoothed by lyspeq's py/smbivspline.py between iterations).

The smoothing step exchanges the estimate through text with seven
significant digits, as the reference does; identical FP64 inputs print
identically, so the FP64 loop agrees with the reference to 1e-9.  CPU tests:
the smoothing and the convergence test against the reference's rules."""
import numpy as np
import pytest

import golden_cases as G
from lyspeq_gb300 import estimator as E


def test_smoothing_matches_scipy_spline_rules():
    rng = np.random.Generator(np.random.PCG64(3))
    z = np.repeat([2.2, 2.4, 2.6], 20)
    k = np.tile(np.linspace(1e-3, 3.9e-2, 20), 3)
    p = 20 * np.exp(-k / 0.02) + rng.normal(0, 0.1, size=60)
    e = np.full(60, 0.1)
    sm = E.smooth_power(z, k, p, e)
    assert sm.shape == p.shape and np.all(np.isfinite(sm))
    assert np.sqrt(np.mean((sm - 20 * np.exp(-k / 0.02)) ** 2)) < 0.1
    sml = E.smooth_power(z, k, np.abs(p), e, interp_log=True)
    assert np.all(sml > 0)


def test_convergence_test_rules():
    f = np.diag([4.0, 1.0])
    inv = np.diag([0.25, 1.0])
    ok, dp = E.has_converged(np.array([1.0, 2.0]), np.array([1.001, 2.0]), inv, f, 2, 0.01)
    assert ok and np.allclose(dp, [0.001, 0.0])
    ok, _ = E.has_converged(np.array([1.0, 2.0]), np.array([2.0, 3.0]), inv, f, 2, 0.01)
    assert not ok


def test_fiducial_power_is_zero_with_turn_off_baseline():
    """powerSpectrumFiducial returns 0 under TurnOffBaseline, so the estimate
    is theta alone and the smoothing fits it without a fiducial offset."""
    c = G.load("tiny_nosfid")
    assert c.opts["turn_off_sfid"]
    on = E.QuadraticEstimator(None, c.bins)
    off = E.QuadraticEstimator(None, c.bins, turn_off_sfid=True)
    assert (on.pfid > 0).all() and not off.pfid.any()


def test_precomputed_fisher_shape_is_checked():
    c = G.load("tiny_nosfid")
    with pytest.raises(ValueError):
        E.QuadraticEstimator(None, c.bins, precomputed_fisher=np.eye(3))
    E.QuadraticEstimator(None, c.bins, precomputed_fisher=np.eye(c.bins.nkz))


class _SumsOnly:
    """Stands in for an engine run with skip_fisher (PrecomputedFisher): the
    d, b, t sums of a fixture's chunks and a zero Fisher sum; the host solve."""

    def __init__(self, c):
        self.fsum, self.dbt = G.global_sums(c)

    def iterate(self, theta=None, precision=None):
        pass

    def download(self):
        return dict(fisher=np.zeros_like(self.fsum), d=self.dbt[0], b=self.dbt[1], t=self.dbt[2])

    def fisher_solve(self, fsum, dbt):
        from lyspeq_gb300 import lqg
        return lqg.fisher_solve(fsum, dbt)


def test_precomputed_fisher_replaces_the_sum(engine_lib):
    """With the reference's own global Fisher matrix (halved) as the
    PrecomputedFisher file and no Fisher matrices from the chunks, the
    estimate is the reference's (core/quadratic_estimate.cpp:478-483)."""
    c = G.load("desi_sub")
    res = E.QuadraticEstimator(_SumsOnly(c), c.bins, precomputed_fisher=c.g["fisher"]).iterate()
    assert G.rel_err(res.fisher, c.g["fisher"]) < 1e-15
    assert G.rel_err(res.theta, c.g["theta"]) < 1e-9


@pytest.mark.gpu
def test_nr_loop_matches_reference(engine_lib):
    from lyspeq_gb300 import lqg
    c = G.load("tiny_iter")
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg)
    assert (eng.add_chunk_list(c.chunks) == 0).all()
    res = E.QuadraticEstimator(eng, c.bins, number_of_iterations=c.nr["n"]).iterate()
    assert G.rel_err(res.fits, c.nr["fits"]) < 1e-9
    assert G.rel_err(res.theta, c.nr["theta"]) < 1e-9
    assert G.rel_err(res.previous, c.nr["previous"]) < 1e-8
    assert G.rel_err(res.fisher, c.nr["fisher"]) < 1e-9
    assert G.rel_err(res.dbt, c.nr["dbt"]) < 1e-9
    # the mixed path through the same loop
    mix = E.QuadraticEstimator(eng, c.bins, number_of_iterations=c.nr["n"], precision="mixed").iterate()
    assert G.fisher_err(mix.fisher, c.nr["fisher"]) < 1e-5
    eng.close()
