"""Autotuner host logic (no GPU): candidate lengths, selection and the
cache, with stand-in plans and context."""
import json
import os
import re

import pytest

from giwaxsim_gb300 import autotune as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sizes_match_the_instantiated_lengths():
    src = open(os.path.join(ROOT, "giwaxsim_gb300", "csrc", "gw_fft.cuh")).read()
    m = re.search(r"kFftSizes\[\]\s*=\s*\{([^}]*)\}", src)
    assert tuple(int(x) for x in m.group(1).split(",")) == T.FFT_SIZES
    for n in T.FFT_SIZES:
        odd = n
        while odd % 2 == 0:
            odd //= 2
        assert odd in (1, 3, 5)


def test_length_candidates():
    assert T.length_candidates(518) == [640, 768]
    assert T.length_candidates(1161) == [1280, 1536]
    assert T.length_candidates(8192) == [8192]
    assert T.length_candidates(9000) == []


class FakeCtx:
    def __init__(self):
        self.calls = 0

    def device_name(self):
        return "FakeGPU sm_103 x152"

    def synchronize(self):
        pass

    def time_ms(self, fn, reps=1):
        for _ in range(reps):
            fn()
        return self.last_ms


class FakePlan:
    made = []
    FUSED = (1024, 1280)  # lengths with a fused shape

    def __init__(self, ctx, fft_y, fft_z, batch_slices, transform, block_variant,
                 binning="auto"):
        ty, tz = transform
        for m, fam in ((fft_y, ty), (fft_z, tz)):
            if fam == "fused" and m and m not in self.FUSED:
                raise T.N.GwError(T.N.GW_ERR_ARG, "no fused transform")
        if binning == "gather" and "fused" in transform:
            raise T.N.GwError(T.N.GW_ERR_ARG, "no gather with a fused kernel")
        self.ctx = ctx
        self.choice = (fft_y, fft_z, batch_slices, ty, tz, block_variant, binning)
        FakePlan.made.append(self.choice)

    def info(self):
        return dict(Ly=579, Nc=584, Lz=414, Nr=402, batch=102, n_slices=360,
                    My=1280, Mz=1024)

    def set_atoms(self):
        pass

    def execute(self):
        fy, fz, b, ty, tz, v, binning = self.choice
        # pretend: fused rows, Stockham columns, the half batch and block
        # variant 2 are fastest
        row = {1280: 1.4, 1536: 1.9}[fy] * (0.8 if ty == "fused" else 1.0)
        col = {1024: 0.8, 1280: 1.0}[fz] * (1.1 if tz == "fused" else 1.0)
        self.ctx.last_ms = (row + col + (0 if b == 51 else 0.05) + (0 if v == 2 else 0.01)
                            - (0.1 if binning == "gather" else 0.0))

    def capture_graph(self):
        pass

    def close(self):
        pass


def test_tune_picks_fastest_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("GIWAXSIM_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(T.N, "fused_variant_count", lambda: 4)
    ctx = FakeCtx()
    FakePlan.made = []
    make = lambda **kw: FakePlan(ctx, **kw)  # noqa: E731
    best = T.tune(make, 1, smooth=1.5, ctx=ctx)
    assert best == dict(fft_y=1280, fft_z=1024, batch_slices=51,
                        transform=("fused", "auto"), block_variant=2,
                        binning="atomic")
    # the shape probe, the default plan, 1 new row length, 1 new column
    # length, 3 new family pairs, 1 new binning (gather is refused with a
    # fused kernel), 2 new batch sizes, 3 new block shapes
    assert len(FakePlan.made) == 1 + 1 + 1 + 1 + 3 + 1 + 2 + 3
    cache = json.load(open(tmp_path / "tune.json"))
    (entry,) = cache.values()
    assert entry["choice"]["transform"] == ["fused", "auto"]
    assert entry["candidates"] == 13 and entry["ms"] < entry["default_ms"]
    FakePlan.made = []
    assert T.tune(make, 1, smooth=1.5, ctx=ctx) == best
    assert len(FakePlan.made) == 1  # only the shape probe
