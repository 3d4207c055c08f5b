"""CPU tests of the autotuner cache: bucketing of the (kind, triangles, work size) key, the text format of
saved caches (round trip, comments, merge) and the rejection of malformed or invalid entries."""
import pytest


def test_cache_round_trip_and_buckets(R, host_ctx, tmp_path):
    src = tmp_path / "in.txt"
    src.write_text("# comment\n"
                   "0 20 21 0 256 8 0 0.5 0.7\n"
                   "   \n"
                   "2 12 16 0 64 16 0 3.25 4.5\n"
                   "3 24 31 0 128 12 4194304 100.0 120.0\n")
    R.autotune_load(host_ctx, src)
    # 1,310,724 triangles -> bucket 20; 2,097,152 rays -> bucket 21; anything in [2^20, 2^21) matches
    t = R.autotune_lookup(host_ctx, R.TUNE_RAYCAST_CLOSEST, 1310724, 2097152)
    assert t is not None and t["trace_block"] == 256 and t["trace_stack"] == 8 and t["refill"] == R.REFILL_GRID
    assert R.autotune_lookup(host_ctx, R.TUNE_RAYCAST_CLOSEST, (1 << 21) - 1, (1 << 22) - 1) is not None
    assert R.autotune_lookup(host_ctx, R.TUNE_RAYCAST_CLOSEST, 1 << 21, 2097152) is None
    assert R.autotune_lookup(host_ctx, R.TUNE_RAYCAST_ANY, 1310724, 2097152) is None
    b = R.autotune_lookup(host_ctx, R.TUNE_BATCH, 1 << 24, 1 << 31)
    assert b["wave_paths"] == 4194304 and b["trace_block"] == 128
    out = tmp_path / "out.txt"
    R.autotune_save(host_ctx, out)
    rows = [l.split() for l in out.read_text().splitlines() if l and not l.startswith("#")]
    assert sorted(r[:7] for r in rows) == sorted([["0", "20", "21", "0", "256", "8", "0"],
                                                  ["2", "12", "16", "0", "64", "16", "0"],
                                                  ["3", "24", "31", "0", "128", "12", "4194304"]])
    # merge: a later file overrides the entry with the same key
    (tmp_path / "upd.txt").write_text("0 20 21 16 128 12 0 0.4 0.7\n")
    R.autotune_load(host_ctx, tmp_path / "upd.txt")
    t = R.autotune_lookup(host_ctx, R.TUNE_RAYCAST_CLOSEST, 1310724, 2097152)
    assert t["refill"] == 16


@pytest.mark.parametrize("line", ["0 20 21 0 256 8", "0 20 21 0 96 8 0 1 1", "0 20 21 0 128 10 0 1 1",
                                  "9 20 21 0 128 12 0 1 1", "0 20 21 0 128 12 0 1 1 extra", "0 20 21 40 128 12 0 1 1"])
def test_malformed_cache_is_rejected(R, tmp_path, line):
    ctx = R.Context(-1)
    try:
        p = tmp_path / "bad.txt"
        p.write_text(line + "\n")
        with pytest.raises(R.ReinaError) as e:
            R.autotune_load(ctx, p)
        assert e.value.code == R.REINA_ERR_IO
        assert R.autotune_lookup(ctx, R.TUNE_RAYCAST_CLOSEST, 1 << 20, 1 << 21) is None
    finally:
        ctx.close()


def test_tuning_fields_validated(R, host_ctx):
    old = host_ctx.tuning()
    with pytest.raises(R.ReinaError):
        host_ctx.set_tuning(trace_block=96)
    with pytest.raises(R.ReinaError):
        host_ctx.set_tuning(trace_stack=10)
    with pytest.raises(R.ReinaError):
        host_ctx.set_tuning(batch_flags=4)
    with pytest.raises(R.ReinaError):
        host_ctx.set_tuning(wave_lanes=17)
    assert old["wave_lanes"] == R.DEFAULT_WAVE_LANES
    with pytest.raises(R.ReinaError):
        host_ctx.set_tuning(wave_paths=(1 << 26) + 1)
    assert old["wave_paths"] == R.DEFAULT_WAVE_PATHS
    host_ctx.set_tuning(trace_block=256, trace_stack=16, batch_flags=R.BATCH_NO_GRAPHS | R.BATCH_FAIR_SHARE)
    t = host_ctx.tuning()
    assert t["trace_block"] == 256 and t["trace_stack"] == 16 and t["batch_flags"] == 3
    host_ctx.set_tuning(**old)
    assert host_ctx.tuning() == old
