"""Host-side pieces of bench.py that the GPU line depends on: the status / percentile summary
behind `completed_value`, and the served-request stream (c5 and its sustainable-load variant)."""
import numpy as np


def test_status_summary_counts_and_completed_rate():
    import bench
    status = np.array([0, 0, 2, 2, 2, 1, 3, 0], dtype=np.int32)
    substeps = np.arange(8, dtype=np.int32)
    iterations = np.array([5, 5, 5, 7, 9, 0, 20000, 4], dtype=np.int32)
    s = bench.status_summary(status, substeps, iterations, seconds=2.0)
    assert s["status_counts"] == {"OK": 3, "SKIPPED": 1, "LIVELOCK": 3, "MAXITER": 1, "ZERO_DT": 0, "ABORTED": 0}
    assert s["completed_value"] == 1.5  # particles with status OK per second
    assert s["iterations_max"] == 20000 and s["iterations_p50"] == 5.0
    assert s["substeps_p50"] == float(np.percentile(substeps, 50))


def test_served_stream_shape():
    import bench
    reqs = bench.serve_requests(48, 5)
    assert len(reqs) == 48
    sizes = np.array([r["T"].size for r in reqs])
    assert sizes.min() >= 1000 and sizes.max() <= 500000
    assert {r["net"] for r in reqs} <= {14, 86, 87}
    for r in reqs:
        assert r["Y"].shape == (r["net"], r["T"].size)
        if r["net"] == 87:
            assert np.all(r["Y"][86] == 0.5)  # electron fraction
    # the sustainable-load variant: sizes divided by 16, arrivals at the requested rate
    small = bench.serve_requests(200, 7, scale=16, rate=25.0)
    assert max(r["T"].size for r in small) <= 500000 // 16 + 1
    gaps = np.array([r["gap"] for r in small])
    assert 0.7 / 25.0 < gaps.mean() < 1.3 / 25.0
    # same seed, same stream
    again = bench.serve_requests(200, 7, scale=16, rate=25.0)
    assert all(np.array_equal(a["T"], b["T"]) and a["gap"] == b["gap"] for a, b in zip(small, again))
