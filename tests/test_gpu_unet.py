"""The learned warm start's tensor-core kernels on the GPU against numpy."""
import ctypes as C

import numpy as np
import pytest

from picfoam_gb300 import abi, native

pytestmark = pytest.mark.gpu


def to_bf16(a):
    """Round-to-nearest-even BF16 bit patterns of float32 values."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def from_bf16(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


def conv_ref(x, w, relu):
    """3x3x3 same convolution, zero padding; x [Z,Y,X,C], w [27,Co,Ci]."""
    Z, Y, X, Ci = x.shape
    xp = np.zeros((Z + 2, Y + 2, X + 2, Ci))
    xp[1:-1, 1:-1, 1:-1] = x
    out = np.zeros((Z, Y, X, w.shape[1]))
    for t in range(27):
        dz, dy, dx = t // 9, (t // 3) % 3, t % 3
        out += np.einsum("zyxc,oc->zyxo", xp[dz:dz + Z, dy:dy + Y, dx:dx + X], w[t])
    return np.maximum(out, 0) if relu else out


def u16p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint16))


@pytest.mark.parametrize("cin,cout,relu", [(16, 16, 0), (32, 64, 1), (64, 32, 0), (16, 48, 0), (96, 32, 1)])
def test_conv_tc_matches_numpy(gpu, cin, cout, relu):
    lib = native.load()
    rng = np.random.default_rng(cin * 100 + cout)
    Z, Y, X = 8, 8, 16
    x = from_bf16(to_bf16(rng.standard_normal((Z, Y, X, cin)).astype(np.float32)))
    w = from_bf16(to_bf16((rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cin)).astype(np.float32)))
    out = np.zeros((Z * Y * X, cout), np.float32)
    xb, wb = to_bf16(x), to_bf16(w)
    st = lib.picgpu_test_conv3d(X, Y, Z, cin, 0, 0, cout, relu, u16p(xb), None, u16p(wb),
                                out.ctypes.data_as(C.POINTER(C.c_float)))
    assert st == abi.OK
    ref = conv_ref(x.astype(np.float64), w.astype(np.float64), relu).reshape(-1, cout)
    # FP32 accumulation of 27 * cin BF16 products; the ReLU form is rounded to BF16
    tol = 2.0 ** -8 * np.abs(ref) + 1e-4 if relu else 1e-4 * np.abs(ref).max()
    assert np.all(np.abs(out - ref) <= tol)


def test_conv_tc_concat_upsampled_source(gpu):
    lib = native.load()
    rng = np.random.default_rng(7)
    Z, Y, X, c1, c2, cout = 8, 8, 16, 32, 16, 16
    coarse = from_bf16(to_bf16(rng.standard_normal((Z // 2, Y // 2, X // 2, c1)).astype(np.float32)))
    skip = from_bf16(to_bf16(rng.standard_normal((Z, Y, X, c2)).astype(np.float32)))
    w = from_bf16(to_bf16((rng.standard_normal((27, cout, c1 + c2)) / 20).astype(np.float32)))
    up = coarse.repeat(2, 0).repeat(2, 1).repeat(2, 2)
    x = np.concatenate([up, skip], axis=3)
    out = np.zeros((Z * Y * X, cout), np.float32)
    st = lib.picgpu_test_conv3d(X, Y, Z, c1, c2, 1, cout, 0, u16p(to_bf16(coarse)), u16p(to_bf16(skip)),
                                u16p(to_bf16(w)), out.ctypes.data_as(C.POINTER(C.c_float)))
    assert st == abi.OK
    ref = conv_ref(x.astype(np.float64), w.astype(np.float64), 0).reshape(-1, cout)
    assert np.abs(out - ref).max() <= 1e-4 * np.abs(ref).max()
