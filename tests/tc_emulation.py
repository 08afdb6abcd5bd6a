"""numpy emulation of the tensor-core correlation pass (fi_correl_tc.cu), stage by
stage, with the same operand packing, Hermitian separation, weights, power-of-two
scales and hi/lo operand splits; products accumulate in float64 here (float32 on
the tensor cores).  Test infrastructure: it checks the algebra of the kernel on the
CPU and predicts each form's plane error.
"""

from __future__ import annotations

import numpy as np

N = 32
SCALE_P = 6
SCALE_Q = 5


def _bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32)


def _round(a, form):
    a = np.asarray(a, dtype=np.float32)
    if form == "fp16x3":
        return a.astype(np.float16).astype(np.float32)
    return _bf16(a)


def split(a, form):
    """Operand terms of a float32 array: [hi] or [hi, lo]."""
    a = np.asarray(a, dtype=np.float32)
    hi = _round(a, form)
    if form == "bf16x1":
        return [hi]
    lo = _round(a - hi, form)
    return [hi, lo]


def product(a, b, form):
    """a @ b.T with the form's terms (hi hi + hi lo + lo hi), float64 sums."""
    if form is None:
        return np.asarray(a, np.float64) @ np.asarray(b, np.float64).T
    sa, sb = split(a, form), split(b, form)
    out = sa[0].astype(np.float64) @ sb[0].astype(np.float64).T
    if len(sa) > 1:
        out += sa[0].astype(np.float64) @ sb[1].astype(np.float64).T
        out += sa[1].astype(np.float64) @ sb[0].astype(np.float64).T
    return out


def constants():
    """B1 (packed real DFT of a row), B2 (complex DFT on [Re | Im]), B4 (real
    inverse with Hermitian weights), each as [N out][K in]."""
    c = lambda j: np.cos(2 * np.pi * (j % N) / N)  # noqa: E731
    s = lambda j: np.sin(2 * np.pi * (j % N) / N)  # noqa: E731
    B1 = np.empty((32, 32))
    B4 = np.empty((32, 32))
    for n in range(32):
        for k in range(32):
            B1[n, k] = c(n * k) if n <= 16 else -s((n - 16) * k)
            if k <= 16:
                B4[n, k] = (1.0 if k in (0, 16) else 2.0) * c(k * n)
            else:
                B4[n, k] = -2.0 * s((k - 16) * n)
    B2 = np.empty((64, 64))
    for n in range(64):
        for k in range(64):
            j = (n % 32) * (k % 32)
            if k < 32:
                B2[n, k] = c(j) if n < 32 else -s(j)
            else:
                B2[n, k] = s(j) if n < 32 else c(j)
    return B1, B2, B4


def correl_plane(w0, w1, form=None):
    """The kernel's correlation plane (raw lags, before the fftshift layout) of two
    32 x 32 windows (values after the image minimum), equal to
    ``ifft2(conj(F0) F1).real`` with ``F = fft2(w)``, ``F[0,0] = 0``."""
    B1, B2, B4 = constants()
    w = [np.asarray(w0, np.float64), np.asarray(w1, np.float64)]
    e, X = [], []
    for wi in w:
        dev = wi - wi.mean()
        S = float((dev * dev).sum())
        ei = 0 if S == 0 else (np.frexp(S / N**2)[1] + 1) >> 1
        ei = max(ei, np.frexp(np.abs(wi).max())[1] - 15)
        e.append(ei)
        ws = np.ldexp(wi, -ei).astype(np.float32)
        Xi = product(ws, B1, form)               # stage 1: rows r x packed kx
        Xi[:, 0] -= np.ldexp(wi.sum(), -ei - 5)  # DC removal (exact)
        X.append(Xi.astype(np.float32))
    Y = []
    for Xi in X:
        A2 = np.zeros((16, 64), np.float32)      # rows kx', K = [Re r | Im r]
        A2[0, :32], A2[0, 32:] = Xi[:, 0], Xi[:, 16]
        for k in range(1, 16):
            A2[k, :32], A2[k, 32:] = Xi[:, k], Xi[:, 16 + k]
        D2 = product(A2, B2, form).astype(np.float32)  # stage 2
        Y.append(D2[:, :32] + 1j * D2[:, 32:].astype(np.float64))
    Z0, Z1 = Y
    P = np.conj(Z0) * Z1
    mirror = (-np.arange(32)) % 32
    a0 = (Z0[0] + np.conj(Z0[0, mirror])) / 2
    b0 = (Z0[0] - np.conj(Z0[0, mirror])) / 2j
    a1 = (Z1[0] + np.conj(Z1[0, mirror])) / 2
    b1 = (Z1[0] - np.conj(Z1[0, mirror])) / 2j
    p0 = np.conj(a0) * a1
    p0[0] = 0.0
    P[0] = p0 + 1j * (np.conj(b0) * b1)
    P = P * 2.0**-SCALE_P
    A3 = np.concatenate([P.imag, P.real], axis=1).astype(np.float32)
    D3 = product(A3, B2, form).astype(np.float32)     # stage 3: [Im Q | Re Q]
    Q = D3 * np.float32(2.0**-SCALE_Q)
    A4 = np.zeros((32, 32), np.float32)               # rows y, K = k4
    A4[:, :16] = Q[:, 32:].T                          # Re Q (kx' = 0: Q0)
    A4[:, 16:] = Q[:, :32].T                          # Im Q (kx' = 0: Q16)
    c = product(A4, B4, form)                         # stage 4: rows y x x
    return c * 2.0 ** (e[0] + e[1] + SCALE_P + SCALE_Q - 10)


def reference_plane(w0, w1, dtype=np.complex128):
    """``ifft2(conj(F0) F1).real`` with ``F[0,0] = 0`` (raw lags)."""
    real = np.float64 if dtype == np.complex128 else np.float32
    F0 = np.fft.fft2(np.asarray(w0, real))
    F1 = np.fft.fft2(np.asarray(w1, real))
    F0[0, 0] = 0
    F1[0, 0] = 0
    return np.fft.ifft2(np.conj(F0) * F1).real
