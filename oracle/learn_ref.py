"""CPU reference of the learned-proposal network (test infrastructure only).

The network of latticednaorigami_gb300/csrc/ldo_mlp.cu restated in numpy:
input encoding (ldo_learn.h: ldo_learn_input), 64 -> 256 -> 256 -> 256 -> 1
with exact (erf) GELU, the weighted logistic loss over bound / total counts
and its gradient.  With bf16=True the matrix operands (inputs, weights,
activations, back-propagated gradients) are rounded to bf16 as the GPU
kernels round them before the tensor-core products; accumulation is float64
here and fp32 on the GPU, so the two agree to bf16/fp32 rounding, not bitwise.
"""
import numpy as np
from scipy.special import erf

DIN, H = 64, 256
NTYPE, NTB, NCOMBO, NDIRF = 32, 64, 256, 4
INS = NTB * NTYPE * NCOMBO
TABLE = INS + NTB * NDIRF   # insertion entries, then regrowth-direction entries
OFF_W1 = 0
OFF_B1 = OFF_W1 + DIN * H
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * H
OFF_W4 = OFF_B3 + H
OFF_B4 = OFF_W4 + H
NPARAM = OFF_B4 + 1
EPS, EPS_T = 0.05, 0.05
LOGIT_CLAMP = 30.0


def tbin(temp):
    b = int(np.floor(temp - 300.0 + 0.5))
    return min(max(b, 0), NTB - 1)


def table_index(tb, tslot, combo):
    return (tb * NTYPE + tslot) * NCOMBO + combo


def tslot(t):
    return 0 if t <= 0 else 1 + (t - 1) % (NTYPE - 1)


def inputs(idx):
    """Input rows (float32) of table entries idx (ldo_learn_input)."""
    idx = np.asarray(idx, np.int64)
    x = np.zeros((len(idx), DIN), np.float32)
    ins = idx < INS
    r = np.arange(len(idx))[ins]
    k = idx[ins]
    combo = k % NCOMBO
    ts = (k // NCOMBO) % NTYPE
    tb = k // (NCOMBO * NTYPE)
    for o in range(4):
        x[r, 4 * o + ((combo >> (2 * o)) & 3)] = 1.0
    x[r, 16 + ts] = 1.0
    x[r, 48] = ((tb - 35) / np.float32(15.0)).astype(np.float32)
    x[r, 49] = 1.0
    r = np.arange(len(idx))[~ins]
    kk = idx[~ins] - INS
    x[r, kk % NDIRF] = 1.0
    x[r, 48] = (((kk // NDIRF) - 35) / np.float32(15.0)).astype(np.float32)
    x[r, 49] = 1.0
    x[r, 50] = 1.0
    return x


def bf16(a):
    """Round float32 values to bf16 (nearest, ties to even), as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def init_params(seed):
    """The engine's seeded initial parameters (splitmix64 uniforms)."""
    p = np.zeros(NPARAM, np.float32)
    mask = (1 << 64) - 1
    state = [(0x9E3779B97F4A7C15 * (seed + 1)) & mask]

    def nxt():
        state[0] = (state[0] + 0x9E3779B97F4A7C15) & mask
        z = state[0]
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z ^= z >> 31
        return (z >> 11) * 2.0 ** -53

    def fill(off, fi, fo):
        a = np.sqrt(6.0 / (fi + fo))
        for i in range(fi * fo):
            p[off + i] = np.float32((2 * nxt() - 1) * a)

    fill(OFF_W1, DIN, H)
    fill(OFF_W2, H, H)
    fill(OFF_W3, H, H)
    fill(OFF_W4, H, 1)
    return p


def _gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def _gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def _unpack(params):
    p = np.asarray(params, np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(DIN, H)
    W2 = p[OFF_W2:OFF_B2].reshape(H, H)
    W3 = p[OFF_W3:OFF_B3].reshape(H, H)
    return W1, p[OFF_B1:OFF_W2], W2, p[OFF_B2:OFF_W3], W3, p[OFF_B3:OFF_W4], p[OFF_W4:OFF_B4], p[OFF_B4]


def forward(params, idx, bf16_ops=True):
    rnd = (lambda a: bf16(a).astype(np.float64)) if bf16_ops else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3, w4, b4 = _unpack(params)
    x = rnd(inputs(idx))
    z1 = x @ rnd(W1) + b1
    h1 = rnd(_gelu(z1))
    z2 = h1 @ rnd(W2) + b2
    h2 = rnd(_gelu(z2))
    z3 = h2 @ rnd(W3) + b3
    h3 = rnd(_gelu(z3))
    out = h3 @ rnd(w4) + b4
    return out, (x, z1, h1, z2, h2, z3, h3)


def loss_grad(params, idx, cnt_b, cnt_t, bf16=True):
    """Loss sum(cnt_t*softplus(z) - cnt_b*z) / sum(cnt_t) and its gradient."""
    rnd = (lambda a: globals()["bf16"](a).astype(np.float64)) if bf16 else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3, w4, b4 = _unpack(params)
    out, (x, z1, h1, z2, h2, z3, h3) = forward(params, idx, bf16)
    cb = np.asarray(cnt_b, np.float64)
    ct = np.asarray(cnt_t, np.float64)
    norm = ct.sum()
    sp = np.logaddexp(0.0, out)
    loss = float(np.sum(ct * sp - cb * out) / norm)
    dout = (ct / (1.0 + np.exp(-out)) - cb) / norm
    g = np.zeros(NPARAM)
    g[OFF_W4:OFF_B4] = h3.T @ dout
    g[OFF_B4] = dout.sum()
    dz3 = np.outer(dout, rnd(w4)) * _gelu_grad(z3)
    g[OFF_B3:OFF_W4] = dz3.sum(0)
    gz3 = rnd(dz3)
    g[OFF_W3:OFF_B3] = (h2.T @ gz3).ravel()
    dz2 = (gz3 @ rnd(W3).T) * _gelu_grad(z2)
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    gz2 = rnd(dz2)
    g[OFF_W2:OFF_B2] = (h1.T @ gz2).ravel()
    dz1 = (gz2 @ rnd(W2).T) * _gelu_grad(z1)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    gz1 = rnd(dz1)
    g[OFF_W1:OFF_B1] = (x.T @ gz1).ravel()
    return loss, g


def table_weights(params, idx):
    out, _ = forward(params, idx, True)
    return np.exp(np.clip(out, -LOGIT_CLAMP, LOGIT_CLAMP))
