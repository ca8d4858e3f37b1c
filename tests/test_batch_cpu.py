"""Host side of the batched form (no GPU): the seeded domain list."""
import numpy as np

from simuverse_gb300 import generate_domains


def test_generated_domains_follow_the_distribution(native):
    d = generate_domains(256, 42)
    assert d == generate_domains(256, 42)
    assert d != generate_domains(256, 43)
    nx = np.array([x["nx"] for x in d])
    ny = np.array([x["ny"] for x in d])
    assert nx.min() >= 64 and nx.max() <= 1024 and ny.min() >= 64 and ny.max() <= 1024
    a = ny / nx
    assert a.min() >= 0.5 - 0.02 and a.max() <= 2.0 + 0.02
    tau = np.array([x["tau"] for x in d])
    sp = np.array([x["speed"] for x in d])
    assert tau.min() >= 0.55 and tau.max() <= 1.0 and sp.min() >= 0.02 and sp.max() <= 0.1
    n_cav = sum(x["scene"] == "cavity" for x in d)
    assert 90 < n_cav < 166
    # log-uniform sides: about half below the geometric mean 256
    assert 0.3 < np.mean(nx < 256) < 0.7
