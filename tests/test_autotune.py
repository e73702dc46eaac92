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

    def __init__(self, ctx, fft_y, fft_z, batch_slices):
        self.ctx, self.choice = ctx, (fft_y, fft_z, batch_slices)
        FakePlan.made.append(self.choice)

    def info(self):
        return dict(Ly=293, Nc=226, Lz=211, Nr=150, batch=180, n_slices=180)

    def set_atoms(self):
        pass

    def execute(self):
        fy, fz, b = self.choice
        # pretend the power of two along z and the half batch are fastest
        self.ctx.last_ms = fy / 640 + (0.5 if fz == 384 else 0.4) + (0 if b == 90 else 0.1)

    def capture_graph(self):
        pass

    def close(self):
        pass


def test_tune_picks_fastest_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("GIWAXSIM_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    ctx = FakeCtx()
    FakePlan.made = []
    make = lambda **kw: FakePlan(ctx, **kw)  # noqa: E731
    best = T.tune(make, 1, smooth=1.5, ctx=ctx)
    assert best == dict(fft_y=640, fft_z=512, batch_slices=90)
    # the default plan plus 2 x 2 lengths x 2 batch sizes (180 is all slices)
    assert len(FakePlan.made) == 1 + 2 * 2 * 2
    cache = json.load(open(tmp_path / "tune.json"))
    (entry,) = cache.values()
    assert entry["choice"] == best and entry["candidates"] == 8
    FakePlan.made = []
    assert T.tune(make, 1, smooth=1.5, ctx=ctx) == best
    assert len(FakePlan.made) == 1  # only the shape probe
