"""Host-side argument checks of the Python mirror (lyspeq_gb300/lqg.py).

The C ABI takes plain pointers and sizes, so it cannot see the length of a
numpy array; the mirror checks lengths and shapes before any call and raises
ValueError instead of letting the library read past an array.  No context
(and no GPU) is needed: the checks run before the library is called.
"""
import numpy as np
import pytest

from lyspeq_gb300 import lqg


def _engine(nkz=6):
    eng = object.__new__(lqg.Engine)   # no context: only the host-side checks run
    eng.nkz = nkz
    return eng


def test_pixel_arrays_and_offsets_are_checked():
    lam, d, iv = np.linspace(4000, 4100, 10), np.zeros(10), np.ones(10)
    out = lqg.Engine._pixel_arrays(lam, d, iv, [0, 4, 10])
    assert [len(a) for a in out] == [10, 10, 10, 3]
    for bad in ([0, 4, 11], [-1, 4, 10], [0, 6, 4, 10], []):
        with pytest.raises(ValueError):
            lqg.Engine._pixel_arrays(lam, d, iv, bad)
    with pytest.raises(ValueError):
        lqg.Engine._pixel_arrays(lam, d[:9], iv, [0, 9])
    with pytest.raises(ValueError):
        _engine().add_chunks(lam, d, iv, [0, 4, 10], [3000])        # one R per chunk


def test_theta_and_solve_shapes_are_checked():
    eng = _engine(6)
    assert eng._theta(None) is None and len(eng._theta(np.zeros(6))) == 6
    with pytest.raises(ValueError):
        eng.iterate(theta=np.zeros(5))
    with pytest.raises(ValueError):
        eng.iterate_async(theta=np.zeros(7))
    with pytest.raises(ValueError):
        eng.fisher_solve(np.zeros((6, 5)), np.zeros((3, 6)))
    with pytest.raises(ValueError):
        eng.fisher_solve(np.zeros((6, 6)), np.zeros((2, 6)))
    with pytest.raises(ValueError):
        eng.bootstrap([0, 1], 10, solver=np.eye(5))
