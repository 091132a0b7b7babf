"""numpy model of the closure network (24-64-64-64-1, tanh-form GELU) with
the BF16 roundings of the device kernels, shared by the GPU tests."""
import numpy as np

NIN, NH = 24, 64


def bf16(a):
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


def unpack(p):
    o = 0
    out = {}
    for name, shape in (("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NH, NH)),
                        ("b3", (NH,)), ("W4", (NH,)), ("b4", (1,))):
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    assert o == p.size
    return out


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3))
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * 0.7978845608028654 * (1 + 3 * 0.044715 * z * z)


def forward_np(p, x, round_act):
    P = unpack(p)
    W = {k: bf16(P[k]).astype(np.float64) for k in ("W1", "W2", "W3", "W4")}
    r = (lambda a: bf16(a).astype(np.float64)) if round_act else (lambda a: a)
    h = r(x.astype(np.float64))
    zs = []
    for i, (Wk, bk) in enumerate((("W1", "b1"), ("W2", "b2"), ("W3", "b3"))):
        z = h @ W[Wk].T + P[bk].astype(np.float64)
        zs.append(z)
        h = gelu(z)
        if i < 2:
            h = r(h)
    return h @ W["W4"] + float(P["b4"][0]), zs, W
