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


def test_clock_sampler_decodes_nvml_reasons_and_keeps_only_its_samples():
    """The NVML path of bench.ClockSampler: clock-event reason bits map to the names
    the bench line reports (sw_power_cap kept, slowdowns named), the median SM clock
    and the maximum are taken over the samples of the timed region only; without
    NVML or nvidia-smi the line says so instead of inventing a clock."""
    import threading
    import bench
    c = bench.ClockSampler(0)
    c.nvml = ("lib", "handle")                 # as after a successful start()
    c.thread = threading.Thread(target=lambda: None)
    c.thread.start()
    c.rows = [(2070.0, 2070.0, 0x0), (2055.0, 2070.0, 0x4), (1800.0, 2070.0, 0x8 | 0x1)]
    out = c.stop()
    assert out["samples"] == 3 and out["sm_mhz"] == 2055.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert out["source"].startswith("nvml")
    c2 = bench.ClockSampler(0)
    c2.rows = [(2070.0, 2070.0, 0x20 | 0x40 | 0x80)]
    c2.nvml = ("lib", "handle")
    c2.thread = threading.Thread(target=lambda: None)
    c2.thread.start()
    assert c2.stop()["reasons"] == ["hw_power_brake_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]
    c3 = bench.ClockSampler(0)                 # neither NVML nor nvidia-smi started
    assert c3.stop()["reasons"] == ["nvidia-smi unavailable"]
