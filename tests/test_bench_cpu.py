"""bench.py's host-side pieces (no GPU): argument defaults and the peak helpers
every workload calls."""
import sys


def test_bench_defaults_and_peak_helpers(monkeypatch):
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench._args()
    assert a.workload == "learned3d" and a.steps >= 1 and a.warmup >= 3 and a.gpus == 1
    peak, kind = bench._peaks()
    assert peak > 0 and kind in ("measured", "fallback")
    hbm, tflops, kind = bench._peaks_tensor()
    assert hbm > 0 and tflops > 0 and kind in ("measured", "fallback")
    for fn in ("run_gpu", "run_ensemble", "run_learned3d", "run_reference", "run_reference_3d"):
        assert callable(getattr(bench, fn))
