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


def test_step3d_workload_inputs_and_reference_arm(monkeypatch, capsys):
    """The step3d workload's input state (generated by the library, not the oracle)
    equals the oracle's 3D warm bubble, and its reference arm reports the
    reference's 3D step as unavailable."""
    import json
    import numpy as np
    import bench
    from oracle import cases
    from pybella_gb300 import workloads
    st = workloads.bubble_3d_state(17, 9, 17)
    grid, prm, Sol, p2, hn, hc, sf = cases.bubble_3d(17, 9, 17, wind=0.0)
    inner = (slice(2, -2),) * 3
    np.testing.assert_array_equal(st["Sol"].rho[inner], Sol["rho"][inner])
    np.testing.assert_array_equal(st["mpv"].HydroState.rhoY0, hc["rhoY0"])
    np.testing.assert_array_equal(st["mpv"].HydroState_n.S0, hn["S0"])
    assert st["ud"].Msq == prm.Msq and st["ud"].gravity_strength[1] == prm.g
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "step3d", "--impl", "reference"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "cannot run" in line["unavailable"]


def test_step2d_workload_inputs_and_cpu_sample(monkeypatch):
    """The step2d workload's state (generated by the library) equals the oracle's
    rising bubble; its CPU sample runs the oracle's step."""
    import numpy as np
    import bench
    from oracle import cases
    from pybella_gb300 import workloads
    st = workloads.bubble_2d_state()
    grid, prm, Sol, p2, hn, hc, sf = cases.rising_bubble()
    inner = (slice(2, -2), slice(2, -2))
    np.testing.assert_array_equal(st["Sol"].rho[inner], Sol["rho"][inner])
    np.testing.assert_array_equal(st["mpv"].HydroState_n.S0, hn["S0"])
    v, k = bench._cpu_step2d_sample(0.0)
    assert k == 1 and v > 0
