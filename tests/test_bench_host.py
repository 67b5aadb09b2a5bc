"""Host-side logic of bench.py that needs no GPU."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_heaviside_beta_of_an_iteration():
    """The FP64 comparison restarts from a sampled design with beta_every = 0, so it must be
    given the beta the trajectory used at that iteration: the continuation of psf_simp_step
    (beta *= beta_mult at the start of iteration k whenever k % beta_every == 0)."""
    sys.path.insert(0, ROOT)
    import bench
    pr = dict(heaviside=1, beta=0.5, beta_every=40, beta_mult=2.0)
    beta = pr["beta"]
    for k in range(130):
        if k % pr["beta_every"] == 0:
            beta *= pr["beta_mult"]
        assert bench.heaviside_beta_at(pr, k) == beta, k
    assert bench.heaviside_beta_at(dict(pr, beta_every=0), 77) == 0.5
