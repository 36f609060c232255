"""The library's Newton-Raphson update (lqg_fisher_solve_n, host FP64) against
lyspeq's own global results.

Every complete golden fixture holds the reference's halved, symmetric Fisher
matrix, the d, b, t sums, the solver and inverse matrices, theta and whether
the damped solver was taken (OneDQuadraticPowerEstimate::iterate tail,
core/quadratic_estimate.cpp:456-498; stableInvertSym,
mathtools/matrix_helper.cpp:330-358).  The unhalved upper sum the engine
accumulates is twice the halved matrix's upper triangle, which is exact.
"""
import os

import numpy as np
import pytest

import golden_cases as G
from oracle import qmle_port as P
from oracle.refsrc import reference_root


def _complete_cases():
    return [n for n in G.CASES if G.load(n).complete]


@pytest.mark.parametrize("name", _complete_cases())
def test_library_update_matches_reference(engine_lib, name):
    from lyspeq_gb300 import lqg
    c = G.load(name)
    # the condition number of the global Fisher matrix bounds the agreement
    # of two FP64 inversions (LU here, LAPACK dgetrf/dgetri in the reference)
    tol = max(1e-10, 1e-15 * np.linalg.cond(c.g["fisher"]))
    fsum = 2.0 * np.triu(c.g["fisher"])
    g = lqg.fisher_solve(fsum, c.g["dbt"])
    assert np.array_equal(g["fisher"], c.g["fisher"])
    assert g["damped"] == int(c.g["damped"])
    assert G.rel_err(g["solver"], c.g["solver"]) < tol
    assert G.rel_err(g["inverse"], c.g["inverse"]) < tol
    assert G.rel_err(g["theta"], c.g["theta"]) < tol
    # the oracle's restatement of the same step
    o = P.newton_raphson_step(fsum, c.g["dbt"])
    assert G.rel_err(g["theta"], o["theta"]) < tol


def test_damped_solver_branch(engine_lib):
    """A Fisher matrix whose spectrum has a jump above 8 takes the damped
    solver (F^2 + s I)^-1 F, as the restatement does; a zero-diagonal bin
    is held out and comes back as zero."""
    from lyspeq_gb300 import lqg
    rng = np.random.Generator(np.random.PCG64(5))
    n = 12
    # spectrum of the bins in use: ..., 10, 1, 0.05; the empty bin 4 enters
    # the inversion as 1, so the smallest ratio is 1 / 0.05 = 20 > 8
    q, _ = np.linalg.qr(rng.standard_normal((n - 1, n - 1)))
    ev = np.concatenate([np.geomspace(1e4, 1e3, n - 4), [10.0, 1.0, 0.05]])
    used = [i for i in range(n) if i != 4]
    f = np.zeros((n, n))
    f[np.ix_(used, used)] = (q * ev) @ q.T
    fsum = 2.0 * np.triu(f)
    dbt = rng.standard_normal((3, n))
    g = lqg.fisher_solve(fsum, dbt)
    o = P.newton_raphson_step(fsum, dbt)
    assert g["damped"] == 1 == int(o["warn"])
    assert g["solver"][4, 4] == 0 and g["inverse"][4, 4] == 0
    # two FP64 solves of F^2 + s I agree to its condition number
    sq = f.copy()               # F as the solve holds it: fsum halved, symmetric
    sq[4, 4] = 1.0
    tol = 1e-15 * np.linalg.cond(sq @ sq + o["damp"] * np.eye(n))
    assert G.rel_err(g["solver"], o["solver"]) < tol
    assert G.rel_err(g["theta"], o["theta"]) < tol


@pytest.mark.parametrize("ratio,spread", [(8.6, "linear"), (7.4, "linear"), (1.02, "cluster"),
                                          (30.0, "geometric"), (2.0, "geometric")])
def test_damping_decision_of_large_matrices(engine_lib, ratio, spread):
    """From n = 64 up a positive definite F goes through the Lanczos test on
    its Cholesky factor before the full eigenvalue test: the decision must be
    the reference's (damp when the smallest |eigenvalue| is more than 8 below
    the next) on both sides of the threshold, for a flat, a clustered and a
    widely spread spectrum, and the results those of the restatement."""
    from lyspeq_gb300 import lqg
    rng = np.random.Generator(np.random.PCG64(11))
    n = 200
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    if spread == "linear":
        ev = np.linspace(1.0, 100.0, n)
    elif spread == "cluster":
        ev = 1.0 + 1e-3 * rng.random(n)
        ev[-1] = 50.0
    else:
        ev = np.geomspace(1.0, 1e7, n)
    ev = np.sort(ev)
    ev[0] = ev[1] / ratio
    f = (q * ev) @ q.T
    f = 0.5 * (f + f.T)
    fsum = 2.0 * np.triu(f)
    dbt = rng.standard_normal((3, n))
    g = lqg.fisher_solve(fsum, dbt)
    o = P.newton_raphson_step(fsum, dbt)
    assert g["damped"] == int(o["warn"]) == int(ratio > 8)
    tol = 1e-14 * np.linalg.cond(f) ** (2 if ratio > 8 else 1)
    assert G.rel_err(g["theta"], o["theta"]) < max(tol, 1e-10)


@pytest.mark.skipif(not os.path.isdir(reference_root()), reason="reference sources absent")
def test_inverse_matches_the_reference_lu_truth(engine_lib):
    """lyspeq's test_LAPACKE_InvertMatrixLU_2 (tests/cblas_tests.cpp:257-283): the
    496 x 496 symmetric matrix of tests/input/test_symmatrix.txt (indefinite, so
    the solve takes its elimination branch) inverted by the library's solve,
    against tests/truth/truth_inverse_matrix.txt: the reference's allClose
    (1e-5 relative, 1e-8 absolute) and the file's printing (6 significant
    digits, 5e-6 relative) on every nonzero element."""
    from lyspeq_gb300 import lqg
    ref = reference_root()
    a = np.loadtxt(os.path.join(ref, "tests", "input", "test_symmatrix.txt"), skiprows=1)
    t = np.loadtxt(os.path.join(ref, "tests", "truth", "truth_inverse_matrix.txt"), skiprows=1)
    assert a.shape == t.shape == (496, 496)
    inv = lqg.fisher_solve(2.0 * np.triu(a), np.zeros((3, 496)))["inverse"]
    assert np.all(np.abs(inv - t) < 1e-8 + 1e-5 * np.maximum(np.abs(inv), np.abs(t)))
    nz = t != 0
    assert np.max(np.abs(inv - t)[nz] / np.abs(t)[nz]) <= 5e-6 * (1 + 1e-6)


def test_rejects_bad_shapes(engine_lib):
    from lyspeq_gb300 import lqg
    with pytest.raises(ValueError):
        lqg.fisher_solve(np.zeros((3, 4)), np.zeros((3, 3)))
