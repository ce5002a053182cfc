"""Index arithmetic of the packed-symmetric storkm layouts, restated on the CPU.

The GPU kernels `k_elem_sym32` (pf_elem_sym.cu) and `k_elem_sym16`
(pf_elem_h16.cu) walk a 60 x 60 symmetric element matrix stored once per
entry, with lane l (0..29) owning rows l and l+30.  These tests restate each
layout and each walk in float64, with no rounding, and check that:
- every entry of the symmetric matrix is stored exactly once;
- the walk reproduces K p for every row.
The GPU parity tests check the kernels themselves; these pin the layouts
they read.
"""
import numpy as np


def packed_off(i, k):
    """Position of K(i, k) in the FP32 layout (pf_internal.h, packed_off)."""
    s = (k - i + 60) % 60
    if s < 30:
        return 60 * s + i
    if s == 30:
        return 1800 + (i if i < 30 else i - 30)
    return 60 * (60 - s) + k


def random_sym(seed):
    a = np.random.default_rng(seed).standard_normal((60, 60))
    return a + a.T


def test_packed_off_stores_each_entry_once():
    owners = {}
    for i in range(60):
        for k in range(60):
            owners.setdefault(packed_off(i, k), set()).add((min(i, k), max(i, k)))
    assert sorted(owners) == list(range(1830))
    assert all(len(v) == 1 for v in owners.values())


def pack32(K):
    D = np.zeros(1832)
    for i in range(60):
        for k in range(60):
            D[packed_off(i, k)] = K[i, k]
    return D


def walk32(D, p):
    """k_elem_sym32's loop: forward distance d and backward distance 30-d per step."""
    pp = np.concatenate([p, p])                          # p twice, as the kernel's 120-float slot
    out = np.zeros(60)
    for l in range(30):
        Dl = lambda off: D[l + off]
        Dw = lambda off: D[l + 60 + off]                 # entries (l - t) mod 60 for t > l
        f0 = Dl(0) * pp[l]
        f1 = Dl(30) * pp[l + 30]
        g0 = g1 = 0.0
        for d in range(1, 30):
            t = 30 - d
            p0, p1 = pp[l + d], pp[l + 30 + d]
            f0 += Dl(60 * d) * p0                        # K(l, l+d)
            f1 += Dl(60 * d + 30) * p1                   # K(l+30, l+30+d)
            g1 += Dl(60 * t + d) * p0                    # K(l+30, l+d)
            g0 += (Dw if l < t else Dl)(59 * t) * p1     # K(l, l-t)
        d30 = Dl(1800)
        out[l] = f0 + d30 * pp[l + 30] + g0
        out[l + 30] = f1 + d30 * pp[l] + g1
    return out


def test_fp32_diagonal_walk_reproduces_the_product():
    for seed in range(3):
        K = random_sym(seed)
        p = np.random.default_rng(100 + seed).standard_normal(60)
        assert np.allclose(walk32(pack32(K), p), K @ p, rtol=0, atol=1e-12 * np.abs(K).sum())


def pack16(K):
    """The FP16 layout's word structure (pf_elem_h16.cu), values kept in float64:
    words 30 s + m = (D[s][m], D[s][m+30]) for s < 30; diagonal 30 as 30 halves."""
    words = np.zeros((900, 2))
    for s in range(30):
        for m in range(30):
            words[30 * s + m] = (K[m, (m + s) % 60], K[m + 30, (m + 30 + s) % 60])
    d30 = np.array([K[i, i + 30] for i in range(30)])
    return words, d30


def walk16(words, d30, p):
    """k_elem_sym16's loop, with p kept as pairs (p[i], p[i+30 mod 60])."""
    pairs = np.array([(p[i % 60], p[(i + 30) % 60]) for i in range(60)])
    out = np.zeros(60)
    for l in range(30):
        p00 = pairs[l]
        w0 = words[l]
        f0, f1 = w0[0] * p00[0], w0[1] * p00[1]
        g0 = g1 = 0.0
        for d in range(1, 30):
            t = 30 - d
            p0, p1 = pairs[l + d]
            wf = words[30 * d + l]
            f0 += wf[0] * p0                             # K(l, l+d)
            f1 += wf[1] * p1                             # K(l+30, l+30+d)
            wrap = l >= t                                # l + d >= 30
            wb = words[30 * t + (l - t if wrap else l + d)]
            g1 += (wb[1] if wrap else wb[0]) * p0        # K(l+30, l+d)
            g0 += (wb[0] if wrap else wb[1]) * p1        # K(l, l+d+30)
        f0 += d30[l] * p00[1]
        f1 += d30[l] * p00[0]
        out[l] = f0 + g0
        out[l + 30] = f1 + g1
    return out


def test_fp16_word_walk_reproduces_the_product():
    for seed in range(3):
        K = random_sym(10 + seed)
        p = np.random.default_rng(200 + seed).standard_normal(60)
        words, d30 = pack16(K)
        assert np.allclose(walk16(words, d30, p), K @ p, rtol=0, atol=1e-12 * np.abs(K).sum())


def test_fp16_words_hold_each_entry_once():
    seen = np.zeros((60, 60), int)
    for s in range(30):
        for m in range(30):
            for i in (m, m + 30):
                k = (i + s) % 60
                seen[i, k] += 1
                if k != i:
                    seen[k, i] += 1
    for i in range(30):
        seen[i, i + 30] += 1
        seen[i + 30, i] += 1
    assert (seen == 1).all()
