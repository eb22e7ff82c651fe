"""CPU oracle of the charging network (TEST INFRASTRUCTURE ONLY).

The 6 -> 64 -> 64 -> 1 tanh MLP of shark_gb300/csrc/mlp.cu in numpy: forward pass and the
gradient of sum((y - y*)^2)/n with respect to every parameter, with the operands of the five
GEMMs rounded to BF16 (round to nearest even) where the tensor-core kernels round them and
everything else in FP32.  Used by tests/ to check the GPU's forward/backward kernels.

Parameter blob (SHARK_MLP_NBLOB floats): W1[64][16] b1[64] W2[64][64] b2[64] w3[64] b3,
feature mean[6], sd[6], target mean, sd.
"""
import numpy as np

F, KIN, H = 6, 16, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * KIN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAM = OFF_B3 + 1
OFF_XMU = NPARAM
OFF_XSD = OFF_XMU + F
OFF_TMU = OFF_XSD + F
OFF_TSD = OFF_TMU + 1
NBLOB = OFF_TSD + 1


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(blob, dtype=np.float32):
    b = np.asarray(blob, dtype=dtype)
    return dict(W1=b[OFF_W1:OFF_B1].reshape(H, KIN), b1=b[OFF_B1:OFF_W2], W2=b[OFF_W2:OFF_B2].reshape(H, H),
                b2=b[OFF_B2:OFF_W3], w3=b[OFF_W3:OFF_B3], b3=b[OFF_B3], xmu=b[OFF_XMU:OFF_XSD],
                xsd=b[OFF_XSD:OFF_TMU], tmu=b[OFF_TMU], tsd=b[OFF_TSD])


def _f32(x):
    return np.asarray(x, dtype=np.float32)


def _ident(x):
    return np.asarray(x, dtype=np.float64)


def forward(blob, feat, exact=False):
    """Network output t (de-normalised) and the intermediates of the backward pass.  exact:
    FP64 throughout without BF16 rounding (for finite-difference checks of the gradient)."""
    rnd = _ident if exact else bf16
    f32 = _ident if exact else _f32
    p = unpack(blob, np.float64 if exact else np.float32)
    f = f32(feat).reshape(-1, F)
    xn = np.zeros((f.shape[0], KIN), np.float64 if exact else np.float32)
    xn[:, :F] = (f - p["xmu"]) / p["xsd"]
    z1 = f32(rnd(xn).astype(np.float64) @ rnd(p["W1"]).astype(np.float64).T)
    h1 = np.tanh(z1 + p["b1"])
    z2 = f32(rnd(h1).astype(np.float64) @ rnd(p["W2"]).astype(np.float64).T)
    h2 = np.tanh(z2 + p["b2"])
    y = f32(h2.astype(np.float64) @ p["w3"].astype(np.float64) + p["b3"])
    return y * p["tsd"] + p["tmu"], dict(xn=xn, h1=h1, h2=h2, y=y, p=p, rnd=rnd, f32=f32)


def gradient(blob, feat, target, exact=False):
    """(gradient[NPARAM], loss) of sum((y - y*)^2)/n, y* the normalised target."""
    _, c = forward(blob, feat, exact)
    p, bf16, _f32 = c["p"], c["rnd"], c["f32"]
    n = c["y"].shape[0]
    yn = (_f32(target) - p["tmu"]) / p["tsd"]
    err = c["y"] - yn
    dy = _f32(2.0 * err / n)
    h1, h2, xn = c["h1"], c["h2"], c["xn"]
    dz2 = _f32(dy[:, None] * p["w3"][None, :] * (1.0 - h2 * h2))
    g = np.zeros(NPARAM, np.float64)
    g[OFF_B3] = dy.sum(dtype=np.float64)
    g[OFF_W3:OFF_B3] = (dy[:, None].astype(np.float64) * h2).sum(axis=0)
    g[OFF_B2:OFF_W3] = dz2.sum(axis=0, dtype=np.float64)
    dz2b = bf16(dz2).astype(np.float64)
    g[OFF_W2:OFF_B2] = (dz2b.T @ bf16(h1).astype(np.float64)).reshape(-1)     # dW2[j][i]
    dh1 = _f32(dz2b @ bf16(p["W2"]).astype(np.float64))
    dz1 = _f32(dh1 * (1.0 - h1 * h1))
    g[OFF_B1:OFF_W2] = dz1.sum(axis=0, dtype=np.float64)
    gw1 = bf16(dz1).astype(np.float64).T @ bf16(xn).astype(np.float64)        # dW1[j][i]
    gw1[:, F:] = 0.0
    g[OFF_W1:OFF_B1] = gw1.reshape(-1)
    return (g if exact else g.astype(np.float32)), float(np.sum(err.astype(np.float64) ** 2))
