"""bench.py's host-side logic (CPU): the clock record it attaches to every line,
the workload description, the peak it divides by, and the row selection of
--next-rows-only. A run whose clock record shows thermal or hardware slowdown
must be visible as such in the JSON line; sw_power_cap is recorded, not hidden."""

import json

import pytest

import bench


def _line(sm, mx=2070, active="0x0", hw="Not Active", hwt="Not Active", swt="Not Active", cap="Not Active"):
    return f"0, {sm}, {mx}, 900.0, {active}, {hw}, {hwt}, {swt}, {cap}"


def test_clock_summary_clean_run():
    c = bench.Clocks(0)
    c.lines = [_line(2070), _line(2070), _line(2055)]
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 3}


def test_clock_summary_reports_throttle_reasons():
    c = bench.Clocks(0)
    c.lines = [_line(1800, cap="Active"), _line(1500, hwt="Active"), _line(1600, swt="Active"),
               _line(1700, hw="Active"), "garbage", "", "0, [N/A], 2070, 1, 0, a, b, c, d"]
    s = c.summary()
    assert s["samples"] == 4
    assert s["sm_mhz"] == 1650.0
    assert s["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap", "sw_thermal_slowdown"]


def test_clock_summary_unsampled():
    s = bench.Clocks(0).summary()
    assert s["samples"] == 0 and s["reasons"] == ["unsampled"]


def test_workload_and_peak():
    cfg = bench.workload_config("f16", report=True)
    assert cfg["cells"] == 512 * 256 * 64 and cfg["storage"] == "f16"
    assert "report steps" in cfg["workload"] and "no flush" in cfg["l2"]
    peak, kind = bench.peaks()
    assert peak > 1000.0 and kind in ("measured", "fallback")
    json.dumps(cfg)


def test_bytes_per_cell_and_traffic_table():
    assert bench.BYTES_PER_CELL == {"f32": 152, "f16": 76, "bf16": 76, "f64": 304}
    # ncu traffic per launch stays near the algorithmic bytes (no re-reads)
    fluid = 8_337_856
    for (storage, report), traffic in bench.NCU_TRAFFIC.items():
        alg = (bench.BYTES_PER_CELL[storage] + (68 if report else 0)) * fluid
        assert 0.8 * alg < traffic < 1.05 * alg, (storage, report)


def test_next_rows_selection(monkeypatch, capsys):
    monkeypatch.setattr("sys.argv", ["bench.py", "--next-rows-only", "heat,nope"])
    with pytest.raises(SystemExit):
        bench.main()
    assert "unknown rows" in capsys.readouterr().err
    assert set(bench.NEXT_ROWS) == {"heat", "flutter", "fsi", "derived"}


def test_warmup_floor(monkeypatch, capsys):
    monkeypatch.setattr("sys.argv", ["bench.py", "--warmup", "2"])
    with pytest.raises(SystemExit):
        bench.main()
    assert "--warmup must be >= 3" in capsys.readouterr().err
