"""The served-batch timeline analysis (torchtt_gb300.timeline.analyse) on hand-made kernel events."""
from torchtt_gb300.timeline import analyse


def test_concurrency_and_stream_gaps():
    ev = [
        {"ts": 0.0, "dur": 10.0, "args": {"stream": 1}},
        {"ts": 12.0, "dur": 8.0, "args": {"stream": 1}},    # gap 2 us on stream 1
        {"ts": 5.0, "dur": 10.0, "args": {"stream": 2}},    # overlaps both kernels of stream 1
        {"ts": 40.0, "dur": 10.0, "args": {"stream": 2}},   # gap 25 us on stream 2
    ]
    out = analyse(ev)
    assert out["kernels"] == 4
    assert abs(out["span_ms"] - 0.050) < 1e-12
    # busy: [0, 20] and [40, 50] -> 30 us; kernel time 38 us
    assert abs(out["busy_ms"] - 0.030) < 1e-12
    assert abs(out["sum_kernel_ms"] - 0.038) < 1e-12
    assert abs(out["mean_in_flight"] - 38.0 / 30.0) < 1e-12
    # two kernels in flight during [5, 10] and [12, 15]
    assert abs(out["ms_at_concurrency"][2] - 0.008) < 1e-12
    # gaps 2 and 25 us; the nearest-rank percentile below q * (count - 1) picks the smaller one
    assert out["stream_gap_us"]["p50"] == 2.0 and out["stream_gap_us"]["p99"] == 2.0
    assert out["streams"]["1"]["kernels"] == 2
    assert abs(out["streams"]["2"]["busy_frac"] - 20.0 / 45.0) < 1e-12
