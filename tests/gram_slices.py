"""A numpy model of the mixed-precision tensor-core Gram (test checker only).

The device Gram (pypolymlp_gb300/csrc/gram_tc.cu) splits FP32 rows, per
1,024-row segment and column, into four fixed-point BF16 slices
n_k 2^-7k with x = 2^e sum_k n_k 2^-7k + O(2^(e-29)) (max |x| < 2^e,
|n_1| <= 128, |n_2..4| <= 64) and sums the slice products of levels 1-5,
scaled by 2^(e_a + e_b).  This module restates that arithmetic in FP64
so that the tests can check the device result against it (the products are
exact in FP64; the per-level sums differ from the device's FP32/float-float
sums by rounding far below the tolerances used) and can show, on the CPU,
how the choice of scheme decides the outcome of an ill-conditioned fit.
"""

import numpy as np

SEG = 1024
PRODUCTS = [(0, 0), (0, 1), (1, 0), (0, 2), (2, 0), (1, 1), (0, 3), (3, 0), (1, 2), (2, 1), (1, 3), (3, 1), (2, 2)]


def slices(x):
    """The four slices of one segment x (rows x F, FP32 values), each with its
    column's 2^e applied (so that slice products are in absolute units)."""
    x = np.asarray(x, dtype=np.float64)
    mx = np.abs(x).max(axis=0)
    _, e = np.frexp(mx)
    zero = mx == 0
    e = np.where(zero, 0, e)
    u = np.where(zero[None, :], 0.0, np.ldexp(x, 7 - e[None, :]))
    out = []
    for k in range(4):
        n = np.rint(u)
        out.append(np.ldexp(n, (e - 7 * (k + 1))[None, :]))
        u = (u - n) * 128.0
    return out


def gram_slices(x32):
    """X^T X of the sliced rows, levels 1-5, summed in FP64."""
    x32 = np.asarray(x32, dtype=np.float32)
    F = x32.shape[1]
    G = np.zeros((F, F))
    for b in range(0, x32.shape[0], SEG):
        sl = slices(x32[b:b + SEG])
        for i, j in PRODUCTS:
            G += sl[i].T @ sl[j]
    return G


def gram_bf16x3(x32, seg=4096):
    """The plain split x = hi + lo (BF16 each) with hi hi + hi lo + lo hi in FP32
    per 4,096-row segment: the scheme the slices replace."""
    import torch

    x = torch.tensor(np.asarray(x32, dtype=np.float32))
    hi = x.to(torch.bfloat16).float()
    lo = (x - hi).to(torch.bfloat16).float()
    G = np.zeros((x.shape[1],) * 2)
    for b in range(0, x.shape[0], seg):
        h, l = hi[b:b + seg], lo[b:b + seg]
        G += (h.T @ h + h.T @ l + l.T @ h).double().numpy()
    return G
