"""The batched entry points pack their requests with whole-array operations
(pack_requests); the packed records must equal the per-request ones
(make_requests) field by field, including what the pointers point to."""
import numpy as np

import tci_gb300 as T


def _deref(r):
    dims = [r.localdims[k] for k in range(r.L)]
    prm = [r.fparams[k] for k in range(r.nparams)] if r.nparams else []
    opts = tuple(getattr(r.opts, nm) for nm, _ in T.Opts._fields_ if nm != "pad_")
    return (r.L, r.fid, dims, prm, r.nparams, opts)


def test_pack_requests_equals_make_requests():
    rng = np.random.default_rng(4)
    specs = []
    for i in range(300):
        L = int(rng.integers(2, 17))
        d = int(rng.integers(2, 17))
        prm = [*(10 ** rng.uniform(-2, 1, size=3)), *rng.integers(1, d + 1, size=L)]
        specs.append((T.DeviceFunction("served", prm), [d] * L,
                      dict(tolerance=10 ** rng.uniform(-10, -6), maxbonddim=int(rng.choice([32, 64, 128, 256])))))
    specs += [
        (T.DeviceFunction("lorentz"), [3] * 4, dict(tolerance=1e-6)),
        (T.DeviceFunction("qtt1d", [0]), [2] * 5, dict(maxbonddim=7, maxiter=3, seed=5)),
        (T.DeviceFunction("lorentz"), [4] * 3, dict(pivottolerance=1e-5, strictlynested=True)),
        (T.DeviceFunction("lorentz"), [4] * 3, {}),
        (T.DeviceFunction("qtt1d", [0]), np.array([2] * 6), dict(sweepstrategy="forward", normalizeerror=False)),
    ]
    arr, keep = T.make_requests(specs)
    ptr, keep2 = T.pack_requests(specs)
    for i in range(len(specs)):
        assert _deref(arr[i]) == _deref(ptr[i]), i
