"""The shared-memory exchanges of the register-resident window FFT (pypty_gb300/csrc/window_fft.cuh)
are free of bank conflicts: restated on the CPU, every 8-byte store and load of both exchanges,
for W = 64 and 128, touches 16 distinct 8-byte bank pairs in each half-warp (a warp's 8-byte
shared-memory access is served as two half-warps of 128 bytes over 32 four-byte banks), and
round 1's 16-byte accesses (a row's elements 2j, 2j+1 as one word) touch 8 distinct 16-byte bank
quads in each quarter-warp.

The addressing follows WinFFT<W>: x1(r, k1) = r*32 + (k1 ^ ((r & 7) << 1)) for the round-1/round-2
exchange and x2(s, kx) = s*W + (kx ^ ((s & 1) << 3)) for the round-2/round-3 exchange; the thread
ownership of each round is Geo<W>'s (round 1: thread (y, n2); round 2: (k1, m2); round 3: (j1, g)).
The inverse transform uses the same index sets with loads and stores swapped."""
import itertools

import numpy as np
import pytest


def geo(W):
    A = W // 32
    C = 32 // A
    Bq = W // C
    Q = 32 // Bq
    T = W * W // 32
    S3 = T // C
    return A, C, Bq, Q, S3, T


def x1(r, k1):
    return r * 32 + (k1 ^ ((r & 7) << 1))


def x2(W, s, kx):
    return s * W + (kx ^ ((s & 1) << 3))


def exchange_instructions(W):
    """Per (name, loop indices): the float2 index each thread t accesses, as an array over t."""
    A, C, Bq, Q, S3, T = geo(W)
    t = np.arange(T)
    out = []
    # round 1 -> xbuf (thread t owns row r = t; elements 2j, 2j+1 as one 16-byte word)
    for j in range(16):
        for k1 in (2 * j, 2 * j + 1):
            out.append(("x1 store (round 1)", (k1,), np.array([x1(r, k1) for r in t])))
    # xbuf -> round 2: thread (k1 = t % 32, m2 = t / 32) reads rows (Bq*m1 + m2)*A + n2
    k1v, m2v = t % 32, t // 32
    for m1, n2 in itertools.product(range(C), range(A)):
        out.append(("x1 load (round 2)", (m1, n2), np.array([x1((Bq * m1 + m2) * A + n2, k) for k, m2 in zip(k1v, m2v)])))
    # round 2 -> xbuf: row m2*C + j1, column k1 + 32*k2
    for j1, k2 in itertools.product(range(C), range(A)):
        out.append(("x2 store (round 2)", (j1, k2), np.array([x2(W, m2 * C + j1, k + 32 * k2) for k, m2 in zip(k1v, m2v)])))
    # xbuf -> round 3: thread (g = t % S3, j1 = t / S3) reads row m2*C + j1, column g + S3*q
    gv, j1v = t % S3, t // S3
    for q, m2 in itertools.product(range(Q), range(Bq)):
        out.append(("x2 load (round 3)", (q, m2), np.array([x2(W, m2 * C + j, g + S3 * q) for g, j in zip(gv, j1v)])))
    return out


@pytest.mark.parametrize("W", [64, 128])
def test_exchanges_are_conflict_free(W):
    A, C, Bq, Q, S3, T = geo(W)
    for name, idx, addr in exchange_instructions(W):
        assert addr.min() >= 0 and addr.max() < W * W, (name, idx)
        if name.endswith("(round 1)"):
            continue   # 16-byte words: test_round1_words_are_aligned_and_conflict_free
        for half in range(0, T, 16):
            a = addr[half:half + 16]
            pairs = a % 16   # 8-byte bank pair of each float2 index
            assert len(set(pairs.tolist())) == 16, (W, name, idx, half, a.tolist())


@pytest.mark.parametrize("W", [64, 128])
def test_exchanges_are_permutations(W):
    """Each exchange writes every xbuf slot once and reads every slot once (no lost values)."""
    A, C, Bq, Q, S3, T = geo(W)
    by_name = {}
    for name, idx, addr in exchange_instructions(W):
        by_name.setdefault(name, []).append(addr)
    for name, addrs in by_name.items():
        allv = np.concatenate(addrs)
        assert allv.size == W * W and np.unique(allv).size == W * W, name


@pytest.mark.parametrize("W", [64, 128])
def test_round1_words_are_aligned_and_conflict_free(W):
    """Round 1 stores (forward) and loads (inverse) elements 2j and 2j+1 of its row as one 16-byte
    word: they must be adjacent and in order, and a quarter-warp's 8 words in 8 bank quads."""
    A, C, Bq, Q, S3, T = geo(W)
    t = np.arange(T)
    for j in range(16):
        a = np.array([x1(r, 2 * j) for r in t])
        b = np.array([x1(r, 2 * j + 1) for r in t])
        assert np.all(a % 2 == 0) and np.all(b == a + 1), (W, j)
        quads = (a // 2) % 8
        for q0 in range(0, T, 8):
            assert len(set(quads[q0:q0 + 8].tolist())) == 8, (W, j, q0)
