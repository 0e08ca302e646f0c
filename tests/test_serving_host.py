"""The serving workload's arrival process on the host: seeded open-loop Poisson arrivals
(exponential inter-arrival times of mean 1/rate), the large-job fraction, and error-bar
targets log-uniform in their range; the same seed gives the same requests."""
import math

import numpy as np

from slater_stoch_gb300 import serving


def test_arrivals_are_poisson_and_seeded():
    reqs = serving.make_requests(seed=11, rate_per_s=50.0, duration_s=20.0, ng0=3)
    t = np.array([r.arrival_s for r in reqs])
    assert np.all(np.diff(t) > 0) and t[-1] <= 20.0
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(len(reqs) - 1000) < 5 * math.sqrt(1000)      # Poisson count
    assert abs(gaps.mean() - 0.02) < 0.002 and abs(gaps.std() / gaps.mean() - 1.0) < 0.1
    sig = np.array([r.sigma_target for r in reqs])
    assert sig.min() >= 1e-7 and sig.max() <= 1e-5
    ls = np.log10(sig)
    assert abs(ls.mean() + 6.0) < 0.1                        # log-uniform on [-7, -5]
    frac = np.mean([r.label == "large" for r in reqs])
    assert abs(frac - 0.05) < 0.02
    again = serving.make_requests(seed=11, rate_per_s=50.0, duration_s=20.0, ng0=3)
    assert [(r.arrival_s, r.seed, r.nint) for r in again] == [(r.arrival_s, r.seed, r.nint) for r in reqs]


def test_small_systems_have_uneven_sizes():
    rng = np.random.default_rng(2)
    sizes = {serving.small_system(rng, ng0=3).n for _ in range(40)}
    assert min(sizes) >= 4 and max(sizes) <= 22 and len(sizes) >= 3
