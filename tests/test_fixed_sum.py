"""The exact fixed-point sum behind the decomposition-independent global
content (mom5gpu_tracer_content_fixed / mom5gpu_fixed_to_double): value =
sum_i acc[i] * 2^(32 i - 100).  The host conversion must give the double
nearest to that exact value (ties to even) for any accumulators a sum of up to
2^31 column values can produce, and the rank allreduce must add accumulators
exactly.  No GPU is used: the conversion is host code of the library, and
Python's Fraction -> float conversion is correctly rounded."""
import os
import socket
from fractions import Fraction

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from mom5_gb300 import capi, decomp

N = capi.FIXED_CHUNKS


def exact(acc):
    return Fraction(sum(int(a) << (32 * i) for i, a in enumerate(acc)), 1 << 100)


def encode(x):
    """trunc(x * 2^100) in 32-bit chunks, each chunk signed like x."""
    X = int(Fraction(x) * (1 << 100))  # int() truncates toward zero
    s, m = (-1 if X < 0 else 1), abs(X)
    return [s * ((m >> (32 * i)) & 0xFFFFFFFF) for i in range(N)]


@pytest.fixture(scope="module")
def lib():
    from mom5_gb300 import build
    build.build()
    capi.lib()


def test_fixed_to_double_rounds_the_exact_sum(lib):
    rng = np.random.default_rng(11)
    cases = [[0] * N, [1] + [0] * (N - 1), [-1] + [0] * (N - 1)]
    # ties: exactly half an ulp above a 53-bit value, even and odd
    for m in ((1 << 52) + 2, (1 << 52) + 3):
        X = (2 * m + 1) << 60
        cases.append([(X >> (32 * i)) & 0xFFFFFFFF for i in range(N)])
    for _ in range(3000):
        k = rng.integers(1, N + 1)
        acc = [0] * N
        for i in rng.choice(N, size=k, replace=False):
            # partial sums of up to 2^31 chunks of either sign: |acc| < 2^63
            acc[i] = int(rng.integers(-(1 << 62), 1 << 62))
        cases.append(acc)
    for acc in cases:
        got = capi.fixed_to_double(acc)
        want = float(exact(acc))
        assert got == want and np.signbit(got) == np.signbit(want) or (got == 0 and want == 0), (acc, got, want)


def test_chunk_sums_of_many_values_are_exact(lib):
    """Encoded column values of both signs and many magnitudes, summed chunk by
    chunk in two different orders: the same accumulators, and the double of
    the exact sum of the truncated values."""
    rng = np.random.default_rng(3)
    xs = rng.normal(size=4000) * 10.0 ** rng.integers(-20, 30, size=4000)
    a1, a2 = [0] * N, [0] * N
    for x in xs:
        a1 = decomp.add_fixed(a1, encode(x))
    for x in xs[::-1]:
        a2 = decomp.add_fixed(a2, encode(x))
    assert a1 == a2
    total = sum(int(Fraction(x) * (1 << 100)) for x in xs)
    assert capi.fixed_to_double(a1) == float(Fraction(total, 1 << 100))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _allreduce_body(rank, world, port, parts, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ex = decomp.RankExchange(decomp.Layout(8 * world, 8, world, 1), rank, None, None, None)
    results[rank] = ex.allreduce_fixed(parts[rank])
    dist.destroy_process_group()


def test_rank_allreduce_adds_accumulators_exactly():
    world = 3
    rng = np.random.default_rng(5)
    parts = [[int(v) for v in rng.integers(-(1 << 60), 1 << 60, size=N)] for _ in range(world)]
    want = parts[0]
    for p in parts[1:]:
        want = decomp.add_fixed(want, p)
    with mp.Manager() as m:
        results = m.dict()
        mp.spawn(_allreduce_body, args=(world, _free_port(), parts, results), nprocs=world, join=True)
        res = dict(results)
    for r in range(world):
        assert res[r] == want
