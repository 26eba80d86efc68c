"""bench.py's host-side pieces without a GPU: the clock-sample summary, the
per-launch DRAM traffic read from the committed ncu summaries, the peak."""
import bench


def test_clock_summary_reports_median_max_and_active_reasons():
    c = bench.ClockSampler(0)
    row = lambda mhz, cap: ["0", str(mhz), "2070", "1100.5", "0x4", "Not Active", "Not Active",
                            "Not Active", cap]
    c.rows = [row(2070, "Not Active"), row(2055, "Active"), row(2070, "Not Active")]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 3
    assert bench.ClockSampler(0).summary()["reasons"] == ["unsampled"]


def test_profile_traffic_is_at_least_the_algorithmic_bytes():
    n = bench.N_PER_ROUND
    malloc = bench.read_profile_traffic("k_churn_malloc_plain")
    free = bench.read_profile_traffic("k_churn_free_plain")
    assert isinstance(malloc, int) and malloc >= 12 * n      # pointer + payload per request
    assert isinstance(free, int) and free >= 12 * n          # pointer + payload per free
    assert bench.read_profile_traffic("no_such_kernel") is None


def test_hbm_peak_has_a_source():
    peak, source = bench.measured_hbm_peak()
    assert peak > 1000 and ("of measured" in source or "of fallback" in source)
