"""Host-side arithmetic of bench.py's JSON line, on the CPU: the roofline figures of each timed
kernel class (algorithmic bytes per launch over the launch-averaged event time, against the
measured copy bandwidth), the choice of the dominant class, and the row selection of
--only-rows."""
import math

import bench


def test_roofline_per_kernel_and_dominant_class():
    cfg, _ = bench.bench_config("C3", "mixed")
    kinds = {1: (1250, 9.6), 2: (20, 8.2), 3: (20, 10.8), 0: (0, 0.0)}
    roof = bench.roofline(kinds, cfg)
    peak = bench.measured_peaks()["hbm_gbs"]
    assert roof["kernel"] == bench.KERNEL_NAMES[3]  # the largest total time
    for kid, (count, ms) in kinds.items():
        name = bench.KERNEL_NAMES[kid]
        if not count:
            assert name not in roof["timed_kernels"]
            continue
        k = roof["timed_kernels"][name]
        per = bench.algorithmic_bytes(kid, cfg)
        assert math.isclose(k["avg_ms"], ms / count)
        assert math.isclose(k["achieved_gbs"], per / (ms / count * 1e-3) / 1e9)
        assert math.isclose(k["frac"], k["achieved_gbs"] / peak)
    # the projection's bytes: 32 B per tracer and 28 B per node
    assert bench.algorithmic_bytes(3, cfg) == 32.0 * cfg.ntr + 28.0 * (cfg.nx + 1) * (cfg.nz + 1)
    assert roof["traffic"] is not None and roof["peak"] == peak


def test_rows_selection_without_rows_is_empty():
    assert bench.extended_rows(None, []) == {}
    assert set(bench.ROW_NAMES) == {"f-1", "f-2", "f-3", "f-4", "A9"}
