"""The CPU reference of the warm-start U-Net: its backward pass against
finite differences (exact FP64 mode), and its BF16-emulating mode against
the exact mode."""
import ctypes as C

import numpy as np
import pytest

F32P = C.POINTER(C.c_float)
F64P = C.POINTER(C.c_double)


def f32p(a):
    return a.ctypes.data_as(F32P)


def sample(rng, X, Y, Z):
    V = X * Y * Z
    x = np.zeros((V, 2), np.float32)
    x[:, 0] = rng.standard_normal(V)
    x[:, 1] = (rng.random(V) > 0.1).astype(np.float32)
    t = rng.standard_normal(V).astype(np.float32)
    m = x[:, 1].copy()
    return x, t, m


def init_weights(lib, rng):
    n = lib.oracle_unet_param_count()
    defs = [(2, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (96, 32), (32, 32), (48, 16), (16, 16),
            (16, 1)]
    assert n == sum(27 * a * b for a, b in defs)
    w = []
    for ci, co in defs:
        w.append(rng.standard_normal(27 * ci * co) * np.sqrt(2.0 / (27 * ci)))
    return np.concatenate(w).astype(np.float32), defs


def loss_of(lib, w, x, t, m, X, Y, Z):
    g = np.zeros(w.size)
    loss = C.c_double()
    assert lib.oracle_unet_gradients(X, Y, Z, f32p(w), f32p(x), f32p(t), f32p(m), 0, g.ctypes.data_as(F64P),
                                     C.byref(loss)) == 0
    return loss.value, g


def test_reference_gradients_match_finite_differences(oracle_backend):
    lib = oracle_backend.load()
    rng = np.random.default_rng(11)
    X = Y = Z = 8
    w, defs = init_weights(lib, rng)
    x, t, m = sample(rng, X, Y, Z)
    _, g = loss_of(lib, w, x, t, m, X, Y, Z)
    offs = np.cumsum([0] + [27 * a * b for a, b in defs])
    ok = 0
    picks = []
    for l in range(len(defs)):
        # the weight with the largest gradient of each layer (well away from round-off)
        seg = np.abs(g[offs[l]:offs[l + 1]])
        picks.append(offs[l] + int(np.argmax(seg)))
    for i in picks:
        h = np.float32(max(1e-3 * abs(w[i]), 1e-4))
        wp, wm = w.copy(), w.copy()
        wp[i] = w[i] + h
        wm[i] = w[i] - h
        lp, _ = loss_of(lib, wp, x, t, m, X, Y, Z)
        lm, _ = loss_of(lib, wm, x, t, m, X, Y, Z)
        fd = (lp - lm) / (float(wp[i]) - float(wm[i]))
        if abs(fd - g[i]) <= 1e-3 * abs(g[i]) + 1e-9:
            ok += 1
    # a ReLU kink inside the difference interval may spoil one pick
    assert ok >= len(picks) - 1


def test_reference_emulation_close_to_exact(oracle_backend):
    lib = oracle_backend.load()
    rng = np.random.default_rng(5)
    X = Y = Z = 8
    w, _ = init_weights(lib, rng)
    x, _, _ = sample(rng, X, Y, Z)
    out = [np.zeros(X * Y * Z) for _ in range(2)]
    for em in (0, 1):
        assert lib.oracle_unet_forward(X, Y, Z, f32p(w), f32p(x), em, out[em].ctypes.data_as(F64P)) == 0
    err = np.linalg.norm(out[1] - out[0]) / np.linalg.norm(out[0])
    # BF16 keeps 8 significant bits: a few tenths of a percent per stored tensor
    assert 1e-5 < err < 5e-2
