"""The shared-memory bank model that picks the FFT exchange pitches
(bri17gb::exchange_pitch, host code in the CUDA library), checked on CPU.

The model: a line of n points is held by T = n/E threads; between radix
stages each thread writes its butterfly outputs to Stockham positions and
reads back its own natural positions t + T q, with one pad slot per 16
elements.  A warp access costs as many shared-memory wavefronts as the
largest number of distinct 4-byte words that fall in one of the 32 banks.
The pitch is the first of n + n/16 + {0..15} that minimises the total over
every warp, stage and access.  This file restates the model independently
and compares choices; it also pins the pitches the design relies on.
"""
import ctypes
from collections import defaultdict

import pytest

from bri17_gb300 import _lib


def _lib_pitch():
    L = _lib.load()
    try:
        f = getattr(L, "_ZN7bri17gb14exchange_pitchEiiibi")
    except AttributeError:
        pytest.skip("exchange_pitch is not exported under the Itanium C++ name")
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_bool, ctypes.c_int]
    f.restype = ctypes.c_int
    return f


def _stages(n, E):
    """Radices of the engines' stages: E = 8 takes 8s and ends with 4 x 4
    (log2 n = 1 mod 3) or one 4 (2 mod 3); E = 16 takes 16s and ends with the
    remaining power of two; E = 12 (n = 3 * 2^k) takes 4s, one 2 when k is
    odd, and the 3 last."""
    if E == 12:
        k = (n // 3).bit_length() - 1
        return n // 12, [4] * (k // 2) + [2] * (k % 2) + [3]
    e = n.bit_length() - 1
    if E == 8:
        a, b = divmod(e, 3)
        return n // 8, ([8] * (a - 1) + [4, 4]) if b == 1 else [8] * a + ([4] if b == 2 else [])
    return n // 16, [16] * (e // 4) + ([1 << (e % 4)] if e % 4 else [])


def _wavefronts(byte_addrs, csize):
    banks = defaultdict(set)
    for a in byte_addrs:
        for w in range(csize // 4):
            word = a // 4 + w
            banks[word % 32].add(word)
    return max(len(s) for s in banks.values())


def _model_cost(n, lines, pitch, csize, lines_fastest, E):
    T, radices = _stages(n, E)
    nthreads = T * lines
    pad = lambda q: q + (q >> 4)  # noqa: E731

    def where(tid):
        return (tid % lines, tid // lines) if lines_fastest else (tid // T, tid % T)

    total = 0
    for w0 in range(0, nthreads, 32):
        tids = range(w0, min(w0 + 32, nthreads))
        Ns = 1
        for R in radices[:-1]:  # the last stage has no exchange
            for m in range(E // R):
                for r in range(R):
                    addrs = []
                    for tid in tids:
                        line, t = where(tid)
                        j = t + T * m
                        jm = j % Ns
                        addrs.append((line * pitch + pad((j - jm) * R + jm + r * Ns)) * csize)
                    total += _wavefronts(addrs, csize)
            for q in range(E):
                addrs = []
                for tid in tids:
                    line, t = where(tid)
                    addrs.append((line * pitch + pad(t + T * q)) * csize)
                total += _wavefronts(addrs, csize)
            Ns *= R
    return total


def _model_pitch(n, lines, csize, lines_fastest, E):
    base = n + n // 16
    costs = [_model_cost(n, lines, base + d, csize, lines_fastest, E) for d in range(16)]
    return base + costs.index(min(costs))


CASES = [(n, lines, cs, lf, 8)
         for n in (16, 32, 64, 128, 256)
         for lines in (1, 2, 4, 8, 16)
         for cs in (8, 16)
         for lf in (True, False)
         if (n // 8) * lines <= 512]
CASES += [(n, lines, 8, True, 16) for n in (256, 512) for lines in (2, 4, 8, 16)]
CASES += [(n, lines, cs, lf, 12)
          for n in (24, 48, 96, 192)
          for lines in (1, 4, 16)
          for cs in (8, 16)
          for lf in (True, False)
          if (n // 12) * lines <= 256]


@pytest.mark.parametrize("n,lines,csize,lines_fastest,E", CASES)
def test_library_pitch_is_the_models_choice(n, lines, csize, lines_fastest, E):
    f = _lib_pitch()
    assert f(n, lines, csize, lines_fastest, E) == _model_pitch(n, lines, csize, lines_fastest, E)


def test_pitches_the_design_relies_on():
    f = _lib_pitch()
    base = lambda n: n + n // 16  # noqa: E731
    # Strided-axis passes, FP32 complex (8 B), lanes across TB lines first:
    # the lines stagger by 16 / TB slots, so the strided reads are
    # conflict-free (the fixed +1 pitch gave two-way conflicts at TB = 8).
    for n in (128, 256, 512):
        for tb in (4, 8, 16):
            assert f(n, tb, 8, True, 8) == base(n) + 16 // tb
    # Row passes (lanes along a line first) at the benchmark row lengths
    # (half lengths 64 and up, at most four lines per warp): no pad beyond
    # one per 16.  Shorter rows put eight lines in a warp and need one.
    for n in (64, 128, 256, 512):
        for lines in (1, 2, 4, 8):
            assert f(n, lines, 8, False, 8) == base(n)
    assert f(32, 2, 8, False, 8) == base(32) + 2
    # Choices are cached per argument set and stable across calls.
    assert f(128, 8, 8, True, 8) == f(128, 8, 8, True, 8)


def _tile_exchange_costs(n, lines, csize, E=8):
    """Wavefronts of every warp access of the exchanges run inside a staged
    tile laid out [element][lines] (element p of line b at p * lines + b,
    no padding), lanes stepping across the lines first -- the float-pair
    TMA axis-0 pass's in-tile exchanges."""
    T, radices = _stages(n, E)
    nthreads = T * lines
    costs = []
    for w0 in range(0, nthreads, 32):
        tids = range(w0, min(w0 + 32, nthreads))
        Ns = 1
        for R in radices[:-1]:
            for m in range(E // R):
                for r in range(R):
                    addrs = []
                    for tid in tids:
                        line, t = tid % lines, tid // lines
                        j = t + T * m
                        jm = j % Ns
                        addrs.append((((j - jm) * R + jm + r * Ns) * lines + line) * csize)
                    costs.append(_wavefronts(addrs, csize))
            for q in range(E):
                addrs = [((tid // lines + T * q) * lines + tid % lines) * csize for tid in tids]
                costs.append(_wavefronts(addrs, csize))
            Ns *= R
    return costs


def test_in_tile_exchanges_take_the_minimum_wavefronts_where_used():
    """Float pairs (16-byte complex) exchange inside the tile where a tile
    row is 128 bytes (8 lines, n0 = 64 and 128): every warp access there
    takes the 4 wavefronts its 512 bytes need.  With 64-byte rows (4 lines,
    n0 = 256) the first stage's writes fall on half the banks and take 8,
    which is why that length keeps its exchange buffer."""
    for n in (64, 128):
        costs = _tile_exchange_costs(n, 8, 16)
        assert costs and all(c == 4 for c in costs), (n, sorted(set(costs)))
    costs = _tile_exchange_costs(256, 4, 16)
    assert max(costs) == 8 and min(costs) == 4
