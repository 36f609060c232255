"""P1D and the per-element parity of the mixed path.

The mixed path forms d - b - t, the difference P1D rests on, without the
22-bit trace products: b_s + t_s = tr(Q_s C^-1) - (F theta)_s (C^-1 C C^-1 =
C^-1 for the marginalised inverse), and d_s and tr(Q_s C^-1) are accumulated in
double-float arithmetic from the FP64 C^-1 and y.  So P1D, d and d - b - t
meet the 1e-5 bar per element, F per element (normalised by sqrt(F_ii F_jj)),
and b and t each within 1e-5 of the larger of max |b|, max |t| of the chunk.

Where P1D is compared: on the bins measured at 5 sigma or more.  A small set
of chunks has an ill-conditioned global Fisher matrix (a relative Fisher noise
of 1e-6 moves P1D of the 12 echelle-size reference chunks by 2e-2 at 5
sigma), so P1D is checked against lyspeq's own results on the other
fixtures and against the FP64 path (itself within 1e-10 of lyspeq) on 24
echelle-size chunks, at theta = 0 and at theta != 0.
"""
import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _engine(c):
    from lyspeq_gb300 import lqg
    eng = lqg.Engine(c.bins, c.tables, c.nv, c.lenv, c.nzp, c.max_forest_length, cont=c.marg, **c.opts)
    assert (eng.add_chunk_list(c.chunks) == 0).all()
    return eng


@pytest.mark.parametrize("name,precision", [("echelle_sub", "mixed"), ("desi_sub", "mixed"),
                                            ("desi_sub", "mixed_direct"), ("small_cfg", "mixed"),
                                            ("small_cfg", "mixed_direct")])
def test_per_element_parity_with_the_reference(engine_lib, name, precision):
    """(The direct form misses the Fisher bar on the echelle-size chunks, 9e-5:
    its products C^-1 Q_k cancel ~10^3-fold at high signal to noise.)"""
    c = G.load(name)
    eng = _engine(c)
    eng.iterate(precision=precision)
    out = eng.download()
    assert (out["status"] == 0).all()
    for i, (dbt, fis) in enumerate(zip(c.dbt, c.fisher)):
        d, b, t, f = eng.chunk_result(i)
        assert G.elem_err(d, dbt[0]) < TOL, (i, "d")
        assert G.fisher_err(f, fis) < TOL, (i, "F")
        scale = max(np.max(np.abs(dbt[1])), np.max(np.abs(dbt[2])))
        assert np.max(np.abs(b - dbt[1])) < TOL * scale and np.max(np.abs(t - dbt[2])) < TOL * scale, (i, "b t")
        # the combination the estimate uses
        e_ref = dbt[0] - dbt[1] - dbt[2]
        assert np.max(np.abs((d - b - t) - e_ref)) < 1e-8 * np.max(np.abs(dbt[1])), (i, "d - b - t")
    if name != "echelle_sub":
        # the global solution; its Fisher matrix is that of the fixture's chunks
        from lyspeq_gb300 import lqg
        fsum, dbt = G.global_sums(c)
        g_ref = lqg.fisher_solve(fsum, dbt)
        g = eng.fisher_solve(out["fisher"], np.stack([out["d"], out["b"], out["t"]]))
        err, nbins = G.p1d_err(c.bins, g_ref, g, fsum)
        assert nbins > 0 and err < TOL, (err, nbins)
    eng.close()


@pytest.mark.parametrize("theta_scale", [0.0, 0.05])
def test_p1d_matches_the_fp64_path_on_echelle_size_chunks(engine_lib, theta_scale):
    """24 chunks of N 1000-1500 at R 30000-50000 and sigma ~ 0.05, the regime
    where the trace products alone put P1D 4e-5 away (22-bit b and t carried
    into high-k bins whose power is ~100 times below the noise)."""
    from lyspeq_gb300 import lqg, synth
    w = synth.make_workload("echelle_small", n_chunks=24)
    eng = lqg.Engine(w.bins, w.tables, w.nv, w.lenv, w.nzp, w.max_forest_length,
                     cont=(w.cont_logl_order, w.cont_l_order))
    assert (eng.add_chunk_list([(s.wave, s.delta, 1.0 / s.sigma ** 2, s.r_fwhm) for s in w.spectra]) == 0).all()
    pfid = synth.pd13_power(np.tile(w.bins.k_centers, w.bins.nz), np.repeat(w.bins.z_centers, w.bins.nk))
    theta = theta_scale * pfid if theta_scale else None
    eng.iterate(theta=theta, precision="fp64")
    ref = eng.download()
    per = [eng.chunk_result(i) for i in range(eng.size)]
    g_ref = eng.fisher_solve(ref["fisher"], np.stack([ref["d"], ref["b"], ref["t"]]))
    eng.iterate(theta=theta, precision="mixed")
    mix = eng.download()
    g = eng.fisher_solve(mix["fisher"], np.stack([mix["d"], mix["b"], mix["t"]]))
    err, nbins = G.p1d_err(w.bins, g_ref, g, ref["fisher"])
    assert nbins > 5 and err < TOL, (err, nbins)
    assert G.fisher_err(g["fisher"], g_ref["fisher"]) < TOL
    for i in range(eng.size):
        d, b, t, f = eng.chunk_result(i)
        assert G.elem_err(d, per[i][0]) < TOL
        assert G.fisher_err(f, per[i][3]) < TOL
    eng.close()
