"""Host checks of index arithmetic the CUDA kernels rely on (no GPU).

* bench.py parses its command line (the bench contract's entry point).
* The fused tensor-core kernel's producer store layout (csrc/ozaki.cu,
  k_oz_fused, producer warps): lane -> (pair quarter qq, determinant d) and
  the byte offset of the 16-byte core-matrix row each lane writes per slice,
  restated from the kernel's formulas.  The 8 producer warps must cover one
  slice region of a ring slot (2 tiles x 64 rows x 16 pairs x 2 bytes) exactly
  once, the two lanes of a quarter pair must be adjacent (they swap halves
  with a xor-1 shuffle) and hold the same determinant, and every 8-lane phase
  of a warp's 16-byte store must hit 8 distinct 16-byte bank groups.
"""

import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_parses_its_options():
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--help"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    for opt in ("--gpus", "--steps", "--warmup", "--impl", "--taylor16", "--batch",
                "--davidson-norb", "--diag", "--rdm", "--rows"):
        assert opt in r.stdout


KCHUNK = 16          # K columns (pairs) per chunk
KCHUNK_ELEMS = 1024  # one tile's half of a slice region: 64 rows x 16 pairs


def kmajor_offset(row, k, kdim):
    """Element offset of (row, k) in a K-major core-matrix tile (tcgen05.cuh)."""
    return (row >> 3) * (kdim * 8) + (k >> 3) * 64 + (row & 7) * 8 + (k & 7)


def producer_lane(pw, lane):
    """(qq, d, byte offset) of producer warp pw, lane (csrc/ozaki.cu)."""
    qq = ((lane >> 3) & 1) * 2 + (lane & 1)
    d = pw * 8 + (lane >> 4) * 4 + ((lane >> 1) & 3)
    tile, dl = d >> 5, d & 31
    odd = qq & 1
    roff = tile * KCHUNK_ELEMS * 2 + kmajor_offset(2 * dl + odd, 8 * (qq >> 1), KCHUNK) * 2
    return qq, d, roff


def test_producer_rows_cover_a_slice_region_once():
    seen = set()
    for pw in range(8):
        for lane in range(32):
            qq, d, off = producer_lane(pw, lane)
            assert off % 16 == 0
            for byte in range(off, off + 16):
                assert byte not in seen
                seen.add(byte)
    assert seen == set(range(2 * KCHUNK_ELEMS * 2))


@pytest.mark.parametrize("pw", range(8))
def test_producer_pairs_and_bank_phases(pw):
    lanes = [producer_lane(pw, lane) for lane in range(32)]
    for lane in range(32):
        qq, d, _ = lanes[lane]
        pq, pd, _ = lanes[lane ^ 1]
        assert pd == d and pq == qq ^ 1
    assert len({(q, d) for q, d, _ in lanes}) == 32
    for phase in range(4):
        groups = {(off // 16) % 8 for _, _, off in lanes[8 * phase: 8 * phase + 8]}
        assert len(groups) == 8


@pytest.mark.parametrize("NP", [16, 80, 112, 128])
def test_epilogue_stores_every_output_once(NP):
    """Epilogue warps w < 8 of k_oz_fused: TMEM lane quarter w & 3, column
    half w >> 2 (NP / 2 pairs each); TMEM lane = MMA row = 64 * half + 2 det
    + part.  Over one tile pair every (tile half, determinant, part, pair) is
    stored exactly once."""
    cw = NP // 2
    seen = set()
    for w in range(8):
        quarter, cg = w & 3, w >> 2
        for lane in range(32):
            row = 32 * quarter + lane
            half, det, part = row >> 6, (row & 63) >> 1, row & 1
            for c in range(cw):
                key = (half, det, part, cg * cw + c)
                assert key not in seen
                seen.add(key)
    assert len(seen) == 2 * 32 * 2 * NP
