"""Served request loop (continuous batching) over one resident allocator:
Poisson arrivals of vector (push_back with capacity doubling) and queue (32 B
nodes) jobs of one to eight CTAs, admitted as stream slots and arena bytes
free up.  Every job's
result is the same in the mix as alone (integer checksums, exact), vector
checksums equal the host's, jobs overlapped on the device, nothing failed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_serving_results_same_alone_and_in_the_mix():
    import gallatin_gb300 as G
    from gallatin_gb300 import serve
    g = G.Gallatin.generate_on_device(16 << 30, 42)
    try:
        jobs = serve.make_jobs(80, rate=2000.0, seed=5)
        srv = serve.Server(g, slots=16)
        out = srv.run(jobs)
        assert out["failed_mallocs"] == 0 and out["error_word"] == 0, out
        assert out["max_concurrent_jobs"] > 1
        sums = out["checksums"]
        for j in jobs:
            if j["kind"] == serve.JOB_VECTOR and j["n"] <= (1 << 22):
                assert int(sums[j["id"]]) == serve.vector_checksum(j["id"], j["n"])
        subset = [j for j in jobs if j["n"] <= (1 << 21)][:8]
        multi = [j for j in jobs if serve.job_ctas(j["kind"], j["n"]) > 1][:3]
        assert subset and multi
        assert srv.solo_check(subset + multi, sums) == []
        # every malloc and free of every job is in the latency histograms
        lr = out["latency_requests"]
        assert lr["mallocs"] + lr["frees"] == out["ops"]
        assert out["malloc_cycles_p99"] >= out["malloc_cycles_p50"] > 0
        assert out["free_cycles_p99"] >= out["free_cycles_p50"] > 0
        assert out["job_latency_ms_p99"] >= out["job_latency_ms_p50"] > 0
        assert out["job_device_ms_p99"] >= out["job_device_ms_p50"] > 0
    finally:
        g.close()
