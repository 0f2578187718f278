"""Seeded synthetic inputs for the five benchmark configurations.

The reference fills its matrices with unseeded ``rand()`` (source/src/utils.h:14-22,
backup/layout_trans.cu:59-73); these generators replace that with numpy
``default_rng(seed)`` (PCG64) and a fixed draw order so that every run, the
tests and the benchmark see identical bytes:

* Bernoulli(p) bits are ``rng.random(shape) < p``, drawn row-major in float64,
  in row chunks (chunking does not change the stream).
* Integer B is ``rng.integers(-8, 9, (K, N))`` cast to float32.
* N(0,1) is ``rng.standard_normal((K, N), dtype=float32)``.
* BF16 is float32 rounded to nearest-even (``f32_to_bf16_bits``), stored as
  uint16 bit patterns.

Packed words are LSB-first: column 32w+i of a row is bit i of word w.
"""
import math

import numpy as np

CHUNK_ROWS = 1024


def bernoulli_bits(rng, rows, cols, p):
    out = np.empty((rows, cols), dtype=bool)
    for r0 in range(0, rows, CHUNK_ROWS):
        r1 = min(rows, r0 + CHUNK_ROWS)
        out[r0:r1] = rng.random((r1 - r0, cols)) < p
    return out


def pack_bits(bits):
    """bool [M, K] -> uint32 words [M, ceil(K/32)], LSB = lowest column."""
    bits = np.asarray(bits, dtype=bool)
    M, K = bits.shape
    Kw = (K + 31) // 32
    if K != Kw * 32:
        pad = np.zeros((M, Kw * 32), dtype=bool)
        pad[:, :K] = bits
        bits = pad
    by = np.packbits(bits, axis=1, bitorder="little")
    return np.ascontiguousarray(by).view("<u4").astype(np.uint32, copy=False).reshape(M, Kw)


def unpack_bits(words, K):
    words = np.ascontiguousarray(np.asarray(words, dtype="<u4"))
    M = words.shape[0]
    by = words.view(np.uint8).reshape(M, -1)
    return np.unpackbits(by, axis=1, bitorder="little")[:, :K].astype(bool)


def f32_to_bf16_bits(x):
    """float32 -> bfloat16 bit patterns (uint16), round to nearest even.
    NaN stays NaN (quiet); matches torch's float32 -> bfloat16 conversion."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = x.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    nan = np.isnan(x)
    if nan.any():
        rounded = rounded.copy()
        rounded[nan] = ((u[nan] >> 16) | 0x40).astype(np.uint16)
    return rounded


def bf16_bits_to_f32(b):
    b = np.ascontiguousarray(np.asarray(b, dtype=np.uint16))
    return (b.astype(np.uint32) << 16).view(np.float32)


def config1():
    """1024x1024 Bernoulli(0.1) A (seed 0), B 1024x256 integers in [-8, 8] (seed 1)."""
    A = bernoulli_bits(np.random.default_rng(0), 1024, 1024, 0.1)
    B = np.random.default_rng(1).integers(-8, 9, (1024, 256)).astype(np.float32)
    return dict(name="plain_small_1024x1024x256_int", M=1024, K=1024, N=256,
                words=pack_bits(A), B=B, b_dtype="f32")


def clustered_bits(M=8192, K=8192, n_proto=64, p_proto=0.05, p_flip=0.002,
                   seed_proto=2, seed_rows=3):
    """Rows = random prototype copy with independent bit flips."""
    protos = bernoulli_bits(np.random.default_rng(seed_proto), n_proto, K, p_proto)
    rng = np.random.default_rng(seed_rows)
    A = np.empty((M, K), dtype=bool)
    proto_of = np.empty(M, dtype=np.int64)
    for i in range(M):
        idx = int(rng.integers(0, n_proto))
        flips = rng.random(K) < p_flip
        proto_of[i] = idx
        A[i] = protos[idx] ^ flips
    return A, protos, proto_of


def config2(M=8192, K=8192, N=512):
    """Clustered rows: 64 Bernoulli(0.05) prototypes (seed 2), per row a
    prototype index then p=0.002 flips (seed 3); B N(0,1) float32 (seed 4)."""
    A, _, _ = clustered_bits(M, K)
    B = np.random.default_rng(4).standard_normal((K, N), dtype=np.float32)
    return dict(name="clustered_8192x8192x512_f32", M=M, K=K, N=N,
                words=pack_bits(A), B=B, b_dtype="f32")


def block_bits(M=16384, K=16384, tile=32, p_tile=0.3, p_bit=0.8, seed=5):
    rng = np.random.default_rng(seed)
    present = rng.random((M // tile, K // tile)) < p_tile
    A = bernoulli_bits(rng, M, K, p_bit)
    A &= np.repeat(np.repeat(present, tile, axis=0), tile, axis=1)
    return A, present


def config3(M=16384, K=16384, N=2048):
    """Block-structured A: 32x32 tiles present w.p. 0.3, bits inside
    Bernoulli(0.8) (seed 5); B N(0,1) bf16 (seed 6)."""
    A, _ = block_bits(M, K)
    B = np.random.default_rng(6).standard_normal((K, N), dtype=np.float32)
    return dict(name="block_16384x16384x2048_bf16", M=M, K=K, N=N,
                words=pack_bits(A), B=f32_to_bf16_bits(B), b_dtype="bf16")


def config4_problem(i, N=128):
    """Problem i of the batched set: M, K log-uniform in [64, 4096] rounded to
    multiples of 32, density U(0.01, 0.3), B N(0,1) bf16 (seed 7+i)."""
    rng = np.random.default_rng(7 + i)
    M = int(32 * round(math.exp(rng.uniform(math.log(64), math.log(4096))) / 32))
    K = int(32 * round(math.exp(rng.uniform(math.log(64), math.log(4096))) / 32))
    d = float(rng.uniform(0.01, 0.3))
    A = bernoulli_bits(rng, M, K, d)
    B = rng.standard_normal((K, N), dtype=np.float32)
    return dict(M=M, K=K, N=N, density=d, words=pack_bits(A), B=f32_to_bf16_bits(B))


def config4(n_problems=512, N=128):
    return [config4_problem(i, N) for i in range(n_problems)]


def config4_grad(problem, i):
    """Incoming gradient of problem i of the batched set for its backward
    pass: G = dL/dY [M x N] N(0,1) bf16 (seed 100007+i)."""
    G = np.random.default_rng(100007 + i).standard_normal((problem["M"], problem["N"]), dtype=np.float32)
    return f32_to_bf16_bits(G)


def config5(M=4096, K=4096, N=8192):
    """Mask A 4096x4096 Bernoulli(0.1) (seed 8); X, G 4096x8192 N(0,1) bf16
    (seeds 9, 10)."""
    A = bernoulli_bits(np.random.default_rng(8), M, K, 0.1)
    X = np.random.default_rng(9).standard_normal((K, N), dtype=np.float32)
    G = np.random.default_rng(10).standard_normal((M, N), dtype=np.float32)
    return dict(M=M, K=K, N=N, words=pack_bits(A), X=f32_to_bf16_bits(X),
                G=f32_to_bf16_bits(G))


def config_symbolic(M=8192, K=8192, N=8192):
    """Symbolic pass workload: A = the clustered 8192x8192 rows of config2
    (seeds 2, 3), B a K x N bit matrix Bernoulli(0.002) (seed 11)."""
    A, _, _ = clustered_bits(M, K)
    Bm = bernoulli_bits(np.random.default_rng(11), K, N, 0.002)
    return dict(name="symbolic_8192x8192x8192", M=M, K=K, N=N, a_words=pack_bits(A), b_words=pack_bits(Bm))


def config_int8(M=4096, K=4096, N=256, density=0.05):
    """Bit-plane product workload: A int8 M x K, nonzero w.p. 0.05 with values
    uniform over the 255 nonzero int8 values (seed 12); B N(0,1) float32
    (seed 13)."""
    rng = np.random.default_rng(12)
    mask = rng.random((M, K)) < density
    vals = rng.integers(-128, 127, (M, K))  # -128..126, then 0..126 -> 1..127
    A = np.where(mask, vals + (vals >= 0), 0).astype(np.int8)
    B = np.random.default_rng(13).standard_normal((K, N), dtype=np.float32)
    return dict(name="int8_bitplane_4096x4096x256_d0.05", M=M, K=K, N=N, A=A, B=B)


def bits_to_csr(words, M, K):
    """Packed rows -> (row_ptr int32 [M+1], col int32 [nnz]) on the host."""
    dense = unpack_bits(words, K)
    counts = dense.sum(1)
    row_ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    col = np.nonzero(dense)[1].astype(np.int32)
    return row_ptr, col
