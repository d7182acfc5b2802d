"""bench.py's accounting on CPU: the algorithmic bytes behind the roofline and
the headline GB/s, the kernels one step launches, the clip's FLOP model, the
whole-job rate and the DRAM traffic read from the committed ncu summary.

The large configuration: HEALPix nside 256 (12 * 256^2 = 786,432 cells) <->
0.25-degree lon-lat (1440 x 720 = 1,036,800 cells), 4,375,816 nonzeros, 128
FP32 fields, forward + transpose."""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402

NNZ, ND, NS, K = 4_375_816, 12 * 256 * 256, 1440 * 720, 128


def test_step_bytes_large_configuration():
    """Per direction: 8 B per nonzero (FP32 weight + int32 column), the row
    pointers, and every field element of both grids once."""
    fwd, rev = bench.step_bytes(NNZ, ND, NS, K)
    assert (fwd, rev) == (971_647_044, 972_648_516)
    fields = 4 * K * (NS + ND)
    assert fwd == NNZ * 8 + 4 * (ND + 1) + fields and rev == NNZ * 8 + 4 * (NS + 1) + fields
    # BF16 fields halve only the field bytes; FP64 (12 B per nonzero)
    b16 = bench.step_bytes(NNZ, ND, NS, K, elem=2)
    assert fwd - b16[0] == 2 * K * (NS + ND)
    f64 = bench.step_bytes(NNZ, ND, NS, 1, elem=8, wbytes=8)
    assert f64[0] == NNZ * 12 + 4 * (ND + 1) + 8 * (NS + ND)


def test_e2e_copies_are_the_field_bytes():
    """The end-to-end step copies every input field in and every output out:
    4 B x K x (source + destination cells) each way."""
    fwd, rev = bench.step_bytes(NNZ, ND, NS, K)
    h2d = 4 * K * (NS + ND)
    assert h2d == 933_494_784
    assert fwd + rev - h2d == 2 * NNZ * 8 + 4 * (ND + 1) + 4 * (NS + 1) + h2d


def test_launches_per_step():
    """One merge-path launch per 128-field pass and direction, a fixup where the
    direction has cut rows, a zero fill where it has empty rows."""
    info = {"cut_rows": [37, 0], "empty_rows": [0, 0]}
    assert bench.launches_per_step(info, 128, "cell_major") == 3
    assert bench.launches_per_step(info, 256, "cell_major") == 6
    assert bench.launches_per_step({"cut_rows": [1, 2], "empty_rows": [3, 0]}, 130, "cell_major") == 2 * 2 + 2 * 2 + 1
    assert bench.launches_per_step(info, 128, "field_major") == 2


def test_clip_flop_model_and_job_rate():
    # 4 edges x 4 vertices x 8 + 2 stages x 2 crossings x 19 + 2 fan triangles x 36 + 8 + 28
    assert bench.CLIP_FP64_FLOPS_PER_PAIR == 4 * 4 * 8 + 2 * 2 * 19 + (2 * 36 + 8) + 28 == 312
    assert bench.job_rate(1, 2e9, 1.0) == 2000.0
    assert bench.job_rate(4, 2e9, 2.0) == 4000.0


def test_profiled_traffic_is_read_and_near_the_algorithmic_bytes():
    a = argparse.Namespace(layout="cell_major", fields=128, nside=256, dlon=0.25)
    t = bench.profiled_traffic(a)
    assert isinstance(t, int)
    fwd, _ = bench.step_bytes(NNZ, ND, NS, K)
    assert 0.9 < t / fwd < 1.1  # no wasted re-reads in the captured launch
    assert bench.profiled_traffic(argparse.Namespace(layout="cell_major", fields=64, nside=256, dlon=0.25)) is None
