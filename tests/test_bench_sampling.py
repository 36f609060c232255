"""The fixed CPU sample the bench's cpu_baseline and its --impl reference arm
share (bench.stratified_sample / stratified_rate): deterministic, one chunk of
every size group per round, and a rate estimator that recovers the mean cost
of a known population."""
import numpy as np

import golden_cases  # noqa: F401  (puts the repo root on sys.path via conftest)
import bench


def test_sample_is_fixed_and_covers_every_size_group_each_round():
    rng = np.random.Generator(np.random.PCG64(5))
    n_list = np.exp(rng.uniform(np.log(200), np.log(1200), 4096)).astype(int)
    a = bench.stratified_sample(n_list, 16, 4)
    b = bench.stratified_sample(n_list, 16, 4)
    assert a == b and len(a) == 64 and len(set(a)) == 64
    order = np.argsort(n_list, kind="stable")
    group_of = np.empty(len(n_list), dtype=int)
    for g, idx in enumerate(np.array_split(order, 16)):
        group_of[idx] = g
    for r in range(4):
        assert sorted(group_of[a[16 * r:16 * (r + 1)]]) == list(range(16))


def test_stratified_rate_recovers_the_population_mean_cost():
    rng = np.random.Generator(np.random.PCG64(6))
    n_list = np.exp(rng.uniform(np.log(200), np.log(1200), 4096))
    cost = (n_list / 1000.0) ** 3                         # seconds per chunk, ~N^3
    rates = []
    for seed in range(40):
        idx = bench.stratified_sample(n_list, 16, 4, seed=seed)
        rate, rel_se = bench.stratified_rate(cost[idx], 16)
        rates.append(rate)
        assert 0 < rel_se < 0.2
    # the population's chunks/s is 1 / mean cost; the estimator is within a few %
    assert abs(np.mean(rates) * np.mean(cost) - 1.0) < 0.03
