"""gala_modularity_device_static: modularity on the device for callers that
must not allocate device memory (their device memory belongs to their own
pool allocator, or an allocation's synchronisation is not allowed on their
path).  The entry point keeps its scratch in a file-scope device array, so
this test checks it through the C ABI against the existing host entry point
gala_modularity_host, within the 1e-9 the other modularity checks use, on two
calls in a row (the second call must clear what the first left behind).

The file name makes pytest collect it last; it also passes run alone.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("case", ["karate", "karate_heavy", "rmat_weighted"])
def test_static_modularity_matches_host_two_calls(ffi, golden, torch_cuda, case):
    torch = torch_cuda
    if case == "karate":
        g = ffi.Graph.load_bin(os.path.join(golden, "karate.txt.bin"))
    elif case == "karate_heavy":
        # every weight 2^30: m2 = 156 * 2^30 > 2^32, so a community's Tot^2
        # passes 2^64 and the sum of squares needs 128 bits
        k = ffi.Graph.load_bin(os.path.join(golden, "karate.txt.bin"))
        offs, nbr, _ = k.arrays()
        g = ffi.Graph.from_csr(offs, nbr, np.full(nbr.shape[0], 1 << 30, dtype=np.int32))
    else:
        r = ffi.Graph.rmat(14, 120000, seed=13)
        offs, nbr, _ = r.arrays()
        # symmetric weights: w(u,v) = 1 + (u + v) % 5
        rows = np.repeat(np.arange(offs.shape[0] - 1), np.diff(offs))
        w = (1 + (rows + nbr) % 5).astype(np.int32)
        g = ffi.Graph.from_csr(offs, nbr, w)
    offs, nbr, w = g.arrays()
    n = offs.shape[0] - 1
    rng = np.random.default_rng(3)
    d_offs, d_nbr = _dev(torch, offs), _dev(torch, nbr)
    d_w = _dev(torch, w) if w is not None else None
    # two different partitions, one call each, back to back
    parts = [rng.integers(0, max(2, n // 7), n).astype(np.int32), np.arange(n, dtype=np.int32)[::-1].copy()]
    for lab in parts:
        d_lab = _dev(torch, lab)
        q_dev = ffi.modularity_device_static(n, d_offs.data_ptr(), d_nbr.data_ptr(),
                                             d_w.data_ptr() if d_w is not None else None, d_lab.data_ptr())
        q_host = g.modularity(lab)
        assert abs(q_dev - q_host) < 1e-9, (q_dev, q_host)


def test_static_modularity_rejects_oversized_graph(ffi, torch_cuda):
    torch = torch_cuda
    n = (1 << 20) + 1
    d = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    with pytest.raises(ffi.GalaError) as e:
        ffi.modularity_device_static(n, d.data_ptr(), d.data_ptr(), None, d.data_ptr())
    assert e.value.status == 8


def test_static_modularity_rejects_bad_labels_and_weights(ffi, golden, torch_cuda):
    torch = torch_cuda
    g = ffi.Graph.load_bin(os.path.join(golden, "karate.txt.bin"))
    offs, nbr, _ = g.arrays()
    n = offs.shape[0] - 1
    d_offs, d_nbr = _dev(torch, offs), _dev(torch, nbr)
    lab = np.arange(n, dtype=np.int32)
    lab[5] = n  # outside [0, n)
    with pytest.raises(ffi.GalaError) as e:
        ffi.modularity_device_static(n, d_offs.data_ptr(), d_nbr.data_ptr(), None, _dev(torch, lab).data_ptr())
    assert e.value.status == 1
    w = np.ones(nbr.shape[0], dtype=np.int32)
    w[3] = 0  # not positive
    d_w = _dev(torch, w)
    with pytest.raises(ffi.GalaError) as e:
        ffi.modularity_device_static(n, d_offs.data_ptr(), d_nbr.data_ptr(), d_w.data_ptr(),
                                     _dev(torch, np.arange(n, dtype=np.int32)).data_ptr())
    assert e.value.status == 1
    # the scratch is cleared on the next call: a valid call right after agrees
    # with the host entry point again
    lab = np.arange(n, dtype=np.int32) % 4
    q = ffi.modularity_device_static(n, d_offs.data_ptr(), d_nbr.data_ptr(), None, _dev(torch, lab).data_ptr())
    assert abs(q - g.modularity(lab)) < 1e-9
