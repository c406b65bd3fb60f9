"""mg_eigh_batched_noalloc against mg_eigh_batched on the same matrices.

The no-alloc entry point is for hosts that own every byte of device memory
through their own pool allocator and so cannot let a library call cudaMalloc:
it takes the caller's device buffers and keeps its workspace in one static
device array.  This file sorts last so the entry point also runs after every
other GPU test has used the device.  Two consecutive calls, each at the
workspace limit (nb * ld * ld = 65536: 4 matrices at ld = 128), must agree
with the allocating entry point (eigenvalues within 1e-13 |A|, eigenvectors
within 1e-10 after aligning column signs, zero padding in z, info all zero),
and the second call must leave the device's free memory unchanged.  A batch
of 64 small matrices (the nb limit) is compared the same way.
"""
import ctypes as C

import numpy as np
import pytest

from mocca_gb300 import _abi

pytestmark = pytest.mark.gpu


def _pack(mats, ld):
    a = np.zeros((len(mats), ld, ld))
    for b, m in enumerate(mats):
        a[b, :m.shape[0], :m.shape[0]] = m
    return a, np.array([m.shape[0] for m in mats], dtype=np.int32)


def _host(a, n):
    nb, ld, _ = a.shape
    w = np.zeros((nb, ld))
    z = np.zeros((nb, ld, ld))
    st = _abi.load().mg_eigh_batched(nb, n.ctypes.data_as(_abi._I), ld, a.ctypes.data_as(_abi._D),
                                     w.ctypes.data_as(_abi._D), z.ctypes.data_as(_abi._D))
    assert st == 0, st
    return w, z


def _noalloc(torch, a, n, check_free=False):
    nb, ld, _ = a.shape
    da = torch.from_numpy(a).cuda()
    dw = torch.full((nb, ld), 7.0, dtype=torch.float64, device="cuda")
    dz = torch.full((nb, ld, ld), 7.0, dtype=torch.float64, device="cuda")
    info = torch.full((nb,), 5, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    st = _abi.load().mg_eigh_batched_noalloc(
        nb, n.ctypes.data_as(_abi._I), ld, C.c_void_p(da.data_ptr()), C.c_void_p(dw.data_ptr()),
        C.c_void_p(dz.data_ptr()), C.c_void_p(info.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert st == 0, st
    torch.cuda.synchronize()
    if check_free:
        assert torch.cuda.mem_get_info()[0] == free0
    assert not info.cpu().numpy().any()
    return dw.cpu().numpy(), dz.cpu().numpy()


def _compare(mats, n, ref, got):
    (w0, z0), (w1, z1) = ref, got
    for b, m in enumerate(mats):
        k = int(n[b])
        nrm = np.linalg.norm(m)
        assert np.abs(w1[b, :k] - w0[b, :k]).max() <= 1e-13 * nrm
        za, zb = z0[b, :k, :k], z1[b, :k, :k]
        sign = np.where(np.sum(za * zb, axis=0) < 0.0, -1.0, 1.0)
        assert np.abs(za - zb * sign).max() <= 1e-10
        pad = z1[b].copy()
        pad[:k, :k] = 0.0
        assert not pad.any()


def test_noalloc_matches_allocating_entry(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = np.random.default_rng(11)
    ld = 128
    first = []
    for k in (10, 37, 80, 128):
        x = rng.normal(size=(k, k))
        first.append(x + x.T)
    second = []
    for h in (10, 40, 64, 64):
        e = np.sort(rng.uniform(-30, 30, size=h))
        d = rng.normal(scale=1.5, size=(h, h))
        d = 0.5 * (d + d.T)
        second.append(np.block([[np.diag(e), d], [d.T, -np.diag(e)]]))
    for call, mats in enumerate((first, second)):
        a, n = _pack(mats, ld)
        assert int(n.size) * ld * ld == 65536
        _compare(mats, n, _host(a, n), _noalloc(torch, a, n, check_free=call == 1))


def test_noalloc_batch_of_64(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = np.random.default_rng(12)
    mats = []
    for b in range(64):
        k = 4 + (b % 13)
        x = rng.normal(size=(k, k))
        mats.append(x + x.T)
    a, n = _pack(mats, 16)
    _compare(mats, n, _host(a, n), _noalloc(torch, a, n))


def test_noalloc_rejects_oversize(built):
    n = np.full(5, 128, dtype=np.int32)
    st = _abi.load().mg_eigh_batched_noalloc(5, n.ctypes.data_as(_abi._I), 128, C.c_void_p(8),
                                             C.c_void_p(8), C.c_void_p(8), None, None)
    assert st == _abi.MG_ERR_ARG
