"""The batched-rrLU configuration at full size: 4096 matrices (2r)x(2r), r
uniform in [8, 128] (seed 0), Haar U,V with s_k = 10^(-k/4) plus 1e-12 noise,
reltol 1e-10, maxrank 256.  Pivot rows and columns, pivot counts and errors
must be bit-exact against the oracle for every matrix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_rrlu_batch_full_size(T, oracle):
    from tci_gb300 import workloads

    mats = workloads.rrlu_batch(4096, seed=0)
    got = T.rrlu_batched(mats, maxrank=256, reltol=1e-10)
    ref = oracle.rrlu_batched(mats, maxrank=256, reltol=1e-10)
    bad = 0
    for (gr, gc, gk, ge), (rr, rc, rk, re) in zip(got, ref):
        ok = gk == rk and ge == re and np.array_equal(gr - 1, rr) and np.array_equal(gc - 1, rc)
        bad += not ok
    assert bad == 0, f"{bad} of {len(mats)} matrices differ"
    # with reltol 1e-10 the 1e-12 noise keeps most pivots above threshold: ranks
    # are well above the ~40 the singular values alone would give
    ks = np.array([g[2] for g in got])
    assert ks.min() >= 16 and ks.max() <= 256
