"""The node tables behind the mixed path's theta term for resolution-matrix
chunks (k_theta_reso_tables + rtab_eval in lyspeq_gb300/csrc/lqg_reso.cu):
G(v) = sum_k theta_k (dk / pi) cos(k_c v) sinc(dk v / 2) on nodes every
h = 1 / (20 k_max) with G and h G', interpolated by cubic Hermite, the node
value kept to double-float and the correction in float.  Checked here in
numpy, on the resolution bench's binning and a random theta, against the
analytic sum the FP64 path evaluates per element (core/chunk_estimate.cpp:444-454):
the error stays below 3e-8 of max |G|, so C's theta term carries about
1e-9 of C.  (The kernels themselves are checked against the FP64 path on the
GPU, tests/test_reso.py.)"""
import numpy as np


def _analytic(v, kc, dk, th):
    x = np.outer(v, dk) / 2.0
    sinc = np.where(np.abs(x) < 1e-4, 1.0 - x * x / 6.0, np.sin(x) / np.where(x == 0, 1.0, x))
    return (np.cos(np.outer(v, kc)) * sinc * (dk / np.pi)) @ th


def _derivative(v, kc, dk, th):
    x = np.outer(v, dk) / 2.0
    xs = np.where(x == 0, 1.0, x)
    sinc = np.where(np.abs(x) < 1e-4, 1.0 - x * x / 6.0, np.sin(x) / xs)
    dsinc = np.where(np.abs(x) < 1e-4, -x / 3.0, (x * np.cos(x) - np.sin(x)) / (xs * xs))
    kv = np.outer(v, kc)
    return ((-kc * np.sin(kv) * sinc + np.cos(kv) * dsinc * dk / 2.0) * (dk / np.pi)) @ th


def test_hermite_node_tables_stay_within_3e_8_of_the_analytic_sum():
    edges = np.linspace(0.0, 0.04, 21)              # 20 linear k bands up to 0.04 s/km
    kc, dk = (edges[1:] + edges[:-1]) / 2, np.diff(edges)
    rng = np.random.Generator(np.random.PCG64(3))
    th = rng.normal(0.0, 1.0, kc.size) * 5.0
    h = 0.05 / edges[-1]
    vmax = 46000.0                                  # the widest chunk of the resolution bench, km/s
    nodes = np.arange(int(np.ceil(vmax / h)) + 4) * h
    g = _analytic(nodes, kc, dk, th)
    g_hi = g.astype(np.float32)
    g_lo = (g - g_hi.astype(np.float64)).astype(np.float32)
    d = (h * _derivative(nodes, kc, dk, th)).astype(np.float32)
    v = rng.uniform(0.0, vmax, 200000)
    v[:5] = [0.0, h / 3, 1e-3, vmax, 1234.5]
    x = v / h
    n = np.minimum(np.floor(x).astype(np.int64), nodes.size - 2)
    t = (x - n).astype(np.float32)
    dG = (g_hi[n + 1] - g_hi[n]) + (g_lo[n + 1] - g_lo[n])
    c2 = np.float32(3.0) * dG - np.float32(2.0) * d[n] - d[n + 1]
    c3 = np.float32(-2.0) * dG + d[n] + d[n + 1]
    corr = t * (d[n] + t * (c2 + t * c3))
    approx = g_hi[n].astype(np.float64) + g_lo[n].astype(np.float64) + corr.astype(np.float64)
    exact = _analytic(v, kc, dk, th)
    err = np.max(np.abs(approx - exact)) / np.max(np.abs(g))
    assert err < 3e-8, err
