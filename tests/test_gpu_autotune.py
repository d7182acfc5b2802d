"""The autotuner: on the first apply of a (device, matrix copy, field type,
field count) it times its candidates -- gathers in flight and blocks per SM of
the merge-path kernel, rows per lane group of the row kernel, entries per
batch of the FP64 row kernel -- keeps the fastest, and appends the choice to
its cache file; a later process reads the file and makes the same choice
without timing.  Every candidate sums the same
entries in the same order, so results do not depend on the choice, nor on the
tuner being on.  Each case runs in a fresh process with its own cache file
(CRG_AUTOTUNE_CACHE) and the choices logged to stderr (CRG_AUTOTUNE_LOG)."""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from crg import Regridder, grids, regrid_
R = Regridder(grids.healpix_grid(32), grids.lonlat_regular(2.0, 2.0), normalize=True)
out = []
for K in (128, 16):
    x = torch.randn((R.shape[1], K), generator=torch.Generator(device="cuda").manual_seed(K), device="cuda")
    for RR, xx in ((R, x), (R.transpose(), torch.randn((R.shape[0], K), device="cuda",
                                                        generator=torch.Generator(device="cuda").manual_seed(K + 1)))):
        y = torch.empty((RR.shape[0], K), device="cuda")
        regrid_(y, RR, xx, dims=1)
        out.append(y.cpu().numpy().ravel())
np.save(sys.argv[2], np.concatenate(out))
"""


def _run(tmp_path, name, **env):
    e = {k: v for k, v in os.environ.items() if k != "CRG_SPMM_PATH"}
    e.update(CRG_AUTOTUNE_LOG="1", **env)
    out = tmp_path / f"{name}.npy"
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT / "conservativeregridding.jl_gb300"), str(out)],
                       env=e, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stderr.splitlines() if l.startswith("crg autotune:")]
    return np.load(out), lines


def test_autotune_measures_persists_and_reloads(cuda, tmp_path):
    cache = tmp_path / "autotune.tsv"
    first, log1 = _run(tmp_path, "first", CRG_AUTOTUNE_CACHE=str(cache))
    measured = [l for l in log1 if l.endswith("ms)") and "measured" in l]
    # the merge-path kernel (128 fields), each direction; 16 fields run the
    # narrow merge-path kernel, which has no candidates to time
    assert sum(" cm_nnz " in l for l in measured) == 2 and not any(" cm_rows " in l for l in measured), log1
    text = cache.read_text().splitlines()
    assert len(text) == 2 and all(len(l.split("\t")) == 3 for l in text)
    choices = {l.split("\t")[0]: l.split("\t")[1] for l in text}

    second, log2 = _run(tmp_path, "second", CRG_AUTOTUNE_CACHE=str(cache))
    assert log2 and all(l.endswith("(cached)") for l in log2), log2
    for l in log2:
        key, choice = l[len("crg autotune: "):-len(" (cached)")].rsplit(" -> ", 1)
        assert choices[key] == choice
    assert len(cache.read_text().splitlines()) == 2  # nothing re-measured
    assert np.array_equal(first, second)

    off, log3 = _run(tmp_path, "off", CRG_AUTOTUNE="0", CRG_AUTOTUNE_CACHE=str(tmp_path / "unused.tsv"))
    assert not log3 and not (tmp_path / "unused.tsv").exists()
    assert np.array_equal(first, off)


def test_autotune_cache_off_keeps_memory_only(cuda, tmp_path):
    home = tmp_path / "home"
    home.mkdir()
    _, log = _run(tmp_path, "mem", CRG_AUTOTUNE_CACHE="off", HOME=str(home), XDG_CACHE_HOME=str(home / "xdg"))
    assert any("measured" in l for l in log)
    assert not any(home.rglob("*.tsv"))


def test_autotune_row_kernel_family(cuda, tmp_path):
    """With CRG_SPMM_PATH=rows the cell-major fields run on the row kernel,
    whose rows per lane group are tuned for each of the applies (128 and 16
    fields, each direction); the results do not depend on the choice."""
    cache = tmp_path / "rows.tsv"
    first, log1 = _run(tmp_path, "rows1", CRG_AUTOTUNE_CACHE=str(cache), CRG_SPMM_PATH="rows")
    measured = [l for l in log1 if l.endswith("ms)") and "measured" in l]
    assert sum(" cm_rows " in l for l in measured) == 4 and len(cache.read_text().splitlines()) == 4, log1
    off, _ = _run(tmp_path, "rows0", CRG_AUTOTUNE="0", CRG_SPMM_PATH="rows")
    assert np.array_equal(first, off)


SCRIPT_F64 = r"""
import sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from crg import Regridder, grids, regrid_
R = Regridder(grids.healpix_grid(32), grids.lonlat_regular(2.0, 2.0), normalize=True)
out = []
g = torch.Generator(device="cuda").manual_seed(3)
for K in (8, 16, 24, 6):  # 2, 4 and 8 lanes per row; 6 fields: no 16-byte vectors
    for RR in (R, R.transpose()):
        x = torch.randn((RR.shape[1], K), generator=g, device="cuda", dtype=torch.float64)
        y = torch.empty((RR.shape[0], K), device="cuda", dtype=torch.float64)
        regrid_(y, RR, x, dims=1)
        out.append(y.cpu().numpy().ravel())
np.save(sys.argv[2], np.concatenate(out))
"""


def test_autotune_fp64_row_candidates_same_bits(cuda, tmp_path):
    """The FP64 row kernel's candidates (entries loaded G at a time, or in
    batches of 8 or 4 with the next batch's indices in flight), each forced
    through the cache file, give the bits of the tuned run."""
    e = {k: v for k, v in os.environ.items() if k != "CRG_SPMM_PATH"}
    e.update(CRG_AUTOTUNE_LOG="1")

    def run(name, cache):
        out = tmp_path / f"{name}.npy"
        r = subprocess.run([sys.executable, "-c", SCRIPT_F64, str(ROOT / "conservativeregridding.jl_gb300"), str(out)],
                           env=dict(e, CRG_AUTOTUNE_CACHE=str(cache)), capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
        return np.load(out), [l for l in r.stderr.splitlines() if l.startswith("crg autotune:")]

    tuned, log = run("tuned", tmp_path / "tuned.tsv")
    keys = [l[len("crg autotune: "):].rsplit(" -> ", 1)[0] for l in log if " cm_f64" in l and "measured" in l]
    # 8, 16, 24 fields (vectors) and 6 (strided), each direction
    assert sum(k.startswith("cm_f64 ") for k in keys) == 6 and sum(k.startswith("cm_f64_strided ") for k in keys) == 2, log
    for v in range(3):
        cache = tmp_path / f"forced{v}.tsv"
        cache.write_text("".join(f"{k}\t{v}\t0\n" for k in keys))
        forced, flog = run(f"forced{v}", cache)
        assert sum(l.endswith(f"-> {v} (cached)") for l in flog) >= 2, flog
        assert np.array_equal(forced, tuned), v
