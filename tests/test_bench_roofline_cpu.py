"""The roofline accounting of bench.py on CPU: algorithmic bytes per launch
of every stage kernel, from the plan sizes of the si-100A workload (crop
403, window 414 x 579, band 583 x 403, real grids, gather binning), worked
out by hand here, and the measured-traffic table's coverage of the plan
shapes the bench runs."""
import bench

# gw_voxel_info of the tuned si-100A plan (real grids, gather binning)
INFO = {"crop": 403, "Ly": 579, "Lz": 414, "Nc": 583, "Nr": 403, "My": 1280,
        "Mz": 1024, "k0": -291, "kz0": -201, "real": 1, "gather": 1}
DARGS = {"num_pixels": 1000, "psis": [0.0] * 91}


def test_f1_columns():
    # real grids: the columns ky >= 0 of the band, from m_zero = -k0 on
    assert bench.f1_columns(INFO) == 583 - 291
    assert bench.f1_columns(dict(INFO, real=0)) == 583


def test_row_and_column_bytes():
    S, nf = 180, 292
    # row: the real window grid read (float32), F1 written (complex64)
    row = bench.algorithmic_bytes("row_czt", INFO, None, S, DARGS, 403)
    assert row == S * 414 * (579 * 4 + nf * 8) == 346_667_040
    # column with gather binning: F1 read, every pixel stored once (float32)
    col = bench.algorithmic_bytes("col_czt_bin", INFO, None, S, DARGS, 403)
    assert col == S * (414 * nf * 8 + 403 * nf * 4)
    # column with atomic binning: F1 read, a float64 read-modify-write of
    # every band pixel
    at = dict(INFO, gather=0, real=0)
    col_at = bench.algorithmic_bytes("col_czt_bin", at, None, S, DARGS, 403)
    assert col_at == S * (414 * 583 * 8 + 403 * 583 * 16)


def test_finalize_and_detector_bytes():
    q3 = 403 ** 3
    binned, nonzero = 130_000_000, 46_000_000
    g = bench.algorithmic_bytes("finalize", INFO, None, 360, DARGS, 403,
                                counted=(nonzero, binned))
    assert g == binned * 4 + q3 * 4
    a = bench.algorithmic_bytes("finalize", dict(INFO, gather=0), None, 360,
                                DARGS, 403, counted=(nonzero, binned))
    assert a == nonzero * 8 + q3 * 4
    d = bench.algorithmic_bytes("detector", INFO, None, 360, DARGS, 403)
    assert d == 91 * 1000 * 1000 * 4 + 1000 * 1000 * 8


def test_shared_roof_counts_every_pass():
    r = bench.shared_roof("row_czt", INFO, 180, 0.5)
    # two window rows per transform, forward and inverse, one read and one
    # write of every point per Stockham pass (16 + 16 + 5: three passes)
    assert r["bytes_per_launch"] == 180 * 207 * 2 * 3 * 1280 * 16
    assert r["unit"] == "TB/s" and 0 < r["frac"] < 10
    c = bench.shared_roof("col_czt_bin", INFO, 180, 0.25)
    assert c["bytes_per_launch"] == 180 * 292 * 2 * bench.fft_passes(1024) * 1024 * 16


def test_traffic_table_covers_the_bench_plans():
    for real in (0, 1):
        for k in ("row_czt", "col_czt_bin"):
            assert ("si-100A", k, 1280, 1024, real) in bench.NCU_TRAFFIC
            assert bench.NCU_TRAFFIC[("si-100A", k, 1280, 1024, real)] > 0
