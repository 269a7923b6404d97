"""The tcgen05 split-BF16 product of the purification density step (pdg_tc_selftest) against FP64.

X is symmetric with its spectrum in [0, 1], as the purification iterates are.  The tolerances follow the
number of BF16 partial products: k = 1 keeps 8 significant bits, k = 3 about 16, k = 6 about 24 (the FP32
accumulation then limits it).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {1: 2e-2, 3: 1e-4, 6: 3e-6}   # max |C - X X| relative to max |X X|


def _product(X, k):
    import torch
    from pdynamo_mirror_gb300 import _native
    L = _native.load()
    x = torch.as_tensor(X, dtype=torch.float32, device="cuda").contiguous()
    c = torch.full_like(x, float("nan"))
    st = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    _native.check(L.pdg_tc_selftest(X.shape[0], k, 0, _native.ptr(x), _native.ptr(c), _native.ptr(st),
                                    _native.stream_handle(torch.cuda.current_stream())), "pdg_tc_selftest")
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    return c.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("n", [16, 40, 96, 128, 131, 144])
def test_split_bf16_product_matches_fp64(n):
    rng = np.random.default_rng(n)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    X = ((Q * rng.uniform(0.0, 1.0, n)) @ Q.T).astype(np.float32)
    X = 0.5 * (X + X.T)
    ref = X.astype(np.float64) @ X.astype(np.float64)
    scale = np.abs(ref).max()
    for k in (1, 3, 6):
        C = _product(X, k)
        err = np.abs(C - ref).max() / scale
        assert err < TOL[k], (n, k, err)
