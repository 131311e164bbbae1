"""Physics and precision studies of the step, run through the Solver API.

Each function runs one of the configurations the solver is specified on,
with seeded synthetic start states (there is no dataset), and returns a dict
of results. ``bench.py --study c2|c3|c5`` prints them as one JSON line.

* ``study_c2``: the LES cylinder at Re 300 (512x256x64, r = 16 at (128, 128),
  U = 0.08, slip z-walls, sponge over the last 32 planes, noise +-1e-3). Drag
  and lift history and the Strouhal number from the spectrum of the lift, as
  tack-lbm's collision_check.py:27-31 computes it (rFFT of the lift after the
  start-up, peak frequency times D/U).
* ``study_c3``: the TRT + Smagorinsky sphere at Re 1000 (768x384x128, r = 24
  at (192, 192, 64), U = 0.06) with FP16 and BF16 deviation storage and FP32
  storage, each against the FP64 run: time-averaged drag and the relative L2
  error of the final and the time-averaged velocity field.
* ``study_c5``: the LES box at Re 3000 with a moving top wall (1024x512x256,
  box 64x64x128 at (256, 256, 128), lid u = 0.05, U = 0.08): FP16 against
  FP32 throughput and drag at full size, and the drag error of FP16 and FP32
  against FP64 on the 256x128x64 downsample of the same flow.
* ``study_collision``: tack-lbm's collision_check.py (collision_check.py:9-31)
  through the drop-in: stability and Strouhal number of bgk/trt/les at
  Re 300, 1000 and 3000 on the default Solver.
* ``study_drag_window``: FP32/FP16/BF16 time-averaged drag against FP64 over
  growing windows, with FP32's own error showing where trajectory divergence
  starts to dominate.

The time-averaged drag is the mean of the drag monitor (Solver.monitors,
lbm.py:649-661) over the second half of the run.
"""

import ctypes
import time

import numpy as np

import lbm


def _history(s, steps, every):
    """Run ``steps`` steps with a report step every ``every``; returns (steps, drag, lift)."""
    t, drag, lift = [], [], []
    done = 0
    while done < steps:
        k = min(every, steps - done)
        s.run(k, report_last=True)
        done += k
        m = s.monitors(k)
        t.append(done)
        drag.append(m["drag"])
        lift.append(m["lift"])
    return np.array(t), np.array(drag), np.array(lift)


def strouhal(lift, every, diameter, u0):
    """Shedding frequency of a lift history sampled every ``every`` steps, as
    St = f D / U: the peak of the Hann-windowed rFFT of the mean-removed
    signal, refined by a parabola through the peak and its neighbours."""
    x = np.asarray(lift, np.float64)
    x = (x - x.mean()) * np.hanning(x.size)
    p = np.abs(np.fft.rfft(x)) ** 2
    k = int(np.argmax(p[1:]) + 1)
    shift = 0.0
    if 1 <= k < p.size - 1:
        a, b, c = np.log(p[k - 1] + 1e-300), np.log(p[k] + 1e-300), np.log(p[k + 1] + 1e-300)
        den = a - 2 * b + c
        shift = 0.5 * (a - c) / den if den != 0 else 0.0
    f = (k + shift) / (x.size * every)  # cycles per step
    return f * diameter / u0


def study_c2(steps=20000, every=10, storage="f32", device=0):
    s = lbm.Solver(512, 256, 64, collision="les", obstacle="cylinder", reynolds=300.0, u0=0.08,
                   diameter=32.0, device=device, lateral="periodic", storage=storage,
                   vertical="slip", obstacle_center=(128.0, 128.0, 32.0), sponge_planes=32,
                   init="random", seed=20240601, rho_sigma=0.0, u_noise=1e-3)
    t0 = time.perf_counter()
    t, drag, lift = _history(s, steps, every)
    wall = time.perf_counter() - t0
    tail = t > steps // 4
    st = strouhal(lift[tail], every, 32.0, 0.08)
    half = t > steps // 2
    return {"study": "c2", "workload": "LES cylinder Re 300, 512x256x64, r 16, slip z, sponge 32",
            "storage": storage, "steps": steps, "report_every": every,
            "strouhal": st, "strouhal_reference": 0.200,
            "strouhal_window_steps": [int(t[tail][0]), int(t[-1])],
            "drag_mean_second_half": float(drag[half].mean()),
            "lift_rms_second_half": float(np.sqrt(np.mean(lift[half] ** 2))),
            "glups_wall": 512 * 256 * 64 * steps / wall / 1e9, "finite": bool(np.isfinite(drag).all())}


def _c3_solver(storage, device, cs):
    return lbm.Solver(768, 384, 128, collision="trt", obstacle="sphere", reynolds=1000.0, u0=0.06,
                      diameter=48.0, device=device, storage=storage, cs=cs,
                      obstacle_center=(192.0, 192.0, 64.0))


def _velocity(s):
    s.sync()
    return np.stack([s.fields[k].numpy.astype(np.float64) for k in ("ux", "uy", "uz")])


def _l2(u, ref, fluid):
    d = (u - ref)[:, fluid]
    return float(np.sqrt(np.sum(d * d) / np.sum(ref[:, fluid] ** 2)))


def study_c3(steps=10000, every=100, storages=("f64", "f32", "f16", "bf16"), cs=0.16, device=0):
    """With Cs = 0.1 this flow diverges near step 2400 from the lbm_init start
    (tau0 = 0.5086) in FP64, FP32 and FP16 alike, so the study runs at the
    reference's default Cs = 0.16. Errors are against the FP64 run: the
    time-averaged drag, and the relative L2 error of the final and of the
    time-averaged (second half) velocity field over the fluid cells."""
    out = {"study": "c3", "workload": f"TRT+Smagorinsky sphere Re 1000, 768x384x128, r 24, Cs {cs}",
           "steps": steps, "report_every": every, "runs": {}}
    ref = None
    for st in storages:
        s = _c3_solver(st, device, cs)
        t0 = time.perf_counter()
        drag, mean_u, count, done = [], None, 0, 0
        while done < steps:
            k = min(every, steps - done)
            s.run(k, report_last=True)
            done += k
            drag.append(s.monitors(k)["drag"])
            if done > steps // 2:
                u = _velocity(s)
                mean_u = u if mean_u is None else mean_u + u
                count += 1
        wall = time.perf_counter() - t0
        drag = np.array(drag)
        cd = float(drag[len(drag) // 2:].mean())
        u = _velocity(s)
        mean_u = mean_u / max(count, 1)
        r = {"drag_mean_second_half": cd, "glups_wall": s.lat.n * steps / wall / 1e9,
             "finite": bool(np.isfinite(drag).all())}
        if st == "f64":
            ref = (u, mean_u, cd, s.mask() == 0)
        else:
            r["drag_rel_err_vs_f64"] = abs(cd - ref[2]) / abs(ref[2])
            r["velocity_l2_rel_err_vs_f64"] = _l2(u, ref[0], ref[3])
            r["mean_velocity_l2_rel_err_vs_f64"] = _l2(mean_u, ref[1], ref[3])
        out["runs"][st] = r
        del s, u, mean_u
    return out


def _c5_solver(storage, n, device):
    """n = 1: the full 1024x512x256 lattice; n = 4: its 256x128x64 downsample."""
    return lbm.Solver(1024 // n, 512 // n, 256 // n, collision="les", obstacle="box", reynolds=3000.0,
                      u0=0.08, diameter=64.0 / n, device=device, storage=storage, lateral="lid",
                      u_lid=0.05, obstacle_center=(256.0 / n, 256.0 / n, 128.0 / n),
                      obstacle_size=(32.0 / n, 32.0 / n, 64.0 / n), init="random", seed=5,
                      rho_sigma=0.0, u_noise=1e-3)


def study_c5(steps=5000, every=100, device=0):
    out = {"study": "c5", "workload": "LES box Re 3000 with moving top wall, 1024x512x256 "
           "(box 64x64x128), downsample 256x128x64", "steps": steps, "report_every": every,
           "full": {}, "downsample": {}}
    for st in ("f32", "f16"):
        s = _c5_solver(st, 1, device)
        s.run(10)
        s.sync()
        s._h.call("lbm_timing", 1)
        s.run(200)
        t = (ctypes.c_double * 7)()
        s._h.call("lbm_timing_read", t)
        s._h.call("lbm_timing", 0)
        ms = t[6] / 200
        solid = int(s.mask().sum())
        bpc = {"f32": 152, "f16": 76}[st]
        t_, drag, _ = _history(s, steps, every)
        half = t_ > steps // 2
        out["full"][st] = {"glups": s.lat.n / (ms * 1e-3) / 1e9, "ms_per_step": ms,
                           "hbm_gbs": bpc * (s.lat.n - solid) / (ms * 1e-3) / 1e9,
                           "drag_mean_second_half": float(drag[half].mean()),
                           "finite": bool(np.isfinite(drag).all())}
        del s
    ref = None
    for st in ("f64", "f32", "f16"):
        s = _c5_solver(st, 4, device)
        t_, drag, _ = _history(s, steps, every)
        half = t_ > steps // 2
        cd = float(drag[half].mean())
        r = {"drag_mean_second_half": cd, "finite": bool(np.isfinite(drag).all())}
        if st == "f64":
            ref = cd
        else:
            r["drag_rel_err_vs_f64"] = abs(cd - ref) / abs(ref)
        out["downsample"][st] = r
        del s
    f32, f16 = out["full"]["f32"], out["full"]["f16"]
    out["full"]["f16_speedup_vs_f32"] = f16["glups"] / f32["glups"]
    out["full"]["f16_drag_rel_diff_vs_f32"] = (abs(f16["drag_mean_second_half"] - f32["drag_mean_second_half"])
                                               / abs(f32["drag_mean_second_half"]))
    return out


def raw_strouhal(lift, every, diameter, u0):
    """collision_check.py's estimator (collision_check.py:27-30): the raw rFFT
    peak of the mean-removed second half of a lift history sampled every
    ``every`` steps, as St = f D / U; returns (St, the grid's bin width)."""
    cl = np.asarray(lift[len(lift) // 2:], np.float64)
    cl = cl - cl.mean()
    spec = np.abs(np.fft.rfft(cl))
    freq = np.fft.rfftfreq(len(cl), d=every)
    k = int(np.argmax(spec[1:]) + 1)
    scale = diameter / u0
    return float(freq[k] * scale), float(freq[1] * scale)


# run lengths (steps) at which collision_check.py's raw estimator is evaluated
# on the long Re 300 histories: their second halves put St on grids of
# 0.1, 0.075, 0.05, 0.0375, 0.03, 0.025 and 0.02 (0.200 is on all but 0.075,
# 0.0375 and 0.03)
RAW_LENGTHS = (6000, 8000, 12000, 16000, 20000, 24000, 30000)


def _collision_run(collision, re, steps, every, device, raw_lengths=()):
    """One collision_check.py run (collision_check.py:12-31): the default Solver
    (384x128x64, cylinder D = 24, U = 0.08, periodic y and z, lbm_init start) at
    Reynolds number ``re``, ``every - 1`` quiet steps and one report step per
    block, monitors(every), stop at the first non-finite drag. The Strouhal
    number is the raw rFFT peak of the mean-removed lift over the second half
    of the history (collision_check.py:27-30), with its bin width, and the
    Hann-windowed, parabola-refined peak of ``strouhal``."""
    s = lbm.Solver(collision=collision, reynolds=float(re), device=device)
    lift, blew_up = [], None
    t0 = time.perf_counter()
    for _ in range(steps // every):
        s.run(every, report_last=True)
        m = s.monitors(every)
        if not np.isfinite(m["drag"]):
            blew_up = s.step_count
            break
        lift.append(m["lift"])
    wall = time.perf_counter() - t0
    r = {"collision": collision, "reynolds": re, "steps": steps, "report_every": every,
         "glups_wall": s.lat.n * s.step_count / wall / 1e9}
    if blew_up is not None:
        r.update(stable=False, diverged_at_step=blew_up)
        return r
    cl = np.array(lift[len(lift) // 2:])
    cl -= cl.mean()
    st_raw, st_bin = raw_strouhal(lift, every, s.diameter, s.u0)
    r.update(stable=True, cl_amplitude=float(np.abs(cl).max()), strouhal_raw=st_raw,
             strouhal_bin=st_bin, strouhal_refined=strouhal(cl, every, s.diameter, s.u0))
    if raw_lengths:
        # what collision_check.py prints when run for n steps: the same
        # deterministic history cut at n
        r["raw_by_steps"] = {str(n): dict(zip(("strouhal_raw", "strouhal_bin"),
                                              raw_strouhal(lift[:n // every], every, s.diameter, s.u0)))
                             for n in raw_lengths if n <= steps}
    return r


def study_collision(steps=8000, every=50, long_steps=30000, device=0):
    """tack-lbm's collision_check.py through the drop-in: bgk/trt/les at
    Re 300, 1000 and 3000 (8000 steps, a report every 50). The reference's
    documented answers (README.md:63-67): St = 0.200 for all three models at
    Re 300, BGK diverges at Re 3000, TRT and LES stay stable. With 8000 steps
    the raw rFFT grid is St = k * 0.075, so Re 300 is also run for
    ``long_steps`` steps (a finer grid)."""
    out = {"study": "collision", "workload": "collision_check.py: default Solver 384x128x64, cylinder D 24, "
           "U 0.08, periodic y and z", "steps": steps, "report_every": every, "runs": []}
    for re in (300, 1000, 3000):
        for coll in ("bgk", "trt", "les"):
            out["runs"].append(_collision_run(coll, re, steps, every, device))
    if long_steps:
        out["long"] = [_collision_run(coll, 300, long_steps, every, device, RAW_LENGTHS)
                       for coll in ("bgk", "trt", "les")]
    runs = {(r["reynolds"], r["collision"]): r for r in out["runs"]}
    out["checks"] = {
        "bgk_diverges_at_re3000": not runs[(3000, "bgk")]["stable"],
        "trt_les_stable_at_re3000": runs[(3000, "trt")]["stable"] and runs[(3000, "les")]["stable"],
        "re300_strouhal_within_one_bin_of_0.200": all(
            r["stable"] and abs(r["strouhal_raw"] - 0.2) <= r["strouhal_bin"] for r in out["runs"]
            if r["reynolds"] == 300),
    }
    if long_steps:
        out["checks"]["re300_long_strouhal_within_one_bin_of_0.200"] = all(
            r["stable"] and abs(r["strouhal_raw"] - 0.2) <= r["strouhal_bin"] for r in out["long"])
    return out


def _drag_history(s, steps, every):
    t, drag = [], []
    done = 0
    while done < steps:
        k = min(every, steps - done)
        s.run(k, report_last=True)
        done += k
        t.append(done)
        drag.append(s.monitors(k)["drag"])
    return np.array(t), np.array(drag)


def study_drag_window(steps=4000, every=10, device=0, cases=("c5_downsample", "c3")):
    """Storage error of the time-averaged drag, measured where it can be seen.

    Each case runs FP64, FP32, FP16 and BF16 storage from the same start state
    with the drag monitor every ``every`` steps. For each window end N (a
    quarter, half, three quarters and all of ``steps``) the time-averaged drag
    over steps (N/2, N] of every storage is compared with FP64's. FP32's own
    error in a window bounds what trajectory divergence (not storage
    precision) contributes there; a window where FP32 agrees with FP64 to
    well under 1e-3 isolates FP16/BF16's storage error.

    * c5_downsample: the LES box at Re 3000 with the moving lid, 256x128x64
      (the 1024x512x256 configuration scaled by 1/4), seeded noise;
    * c3: the TRT + Smagorinsky sphere at Re 1000, 768x384x128, r = 24,
      U = 0.06, Cs = 0.16 (Cs = 0.1 diverges in FP64 too)."""
    out = {"study": "drag_window", "steps": steps, "report_every": every, "cases": {}}
    for case in cases:
        hist = {}
        for st in ("f64", "f32", "f16", "bf16"):
            s = _c5_solver(st, 4, device) if case == "c5_downsample" else _c3_solver(st, device, 0.16)
            t0 = time.perf_counter()
            t, drag = _drag_history(s, steps, every)
            hist[st] = (t, drag, time.perf_counter() - t0)
            del s
        windows = []
        for frac in (0.25, 0.5, 0.75, 1.0):
            n_end = int(round(steps * frac / every)) * every
            sel = (hist["f64"][0] > n_end // 2) & (hist["f64"][0] <= n_end)
            ref = float(hist["f64"][1][sel].mean())
            w = {"window": [n_end // 2 + 1, n_end], "f64_drag": ref}
            for st in ("f32", "f16", "bf16"):
                cd = float(hist[st][1][sel].mean())
                w[f"{st}_drag_rel_err"] = abs(cd - ref) / abs(ref)
            windows.append(w)
        out["cases"][case] = {"windows": windows,
                              "finite": {st: bool(np.isfinite(h[1]).all()) for st, h in hist.items()},
                              "wall_s": {st: h[2] for st, h in hist.items()}}
    return out


STUDIES = {"c2": study_c2, "c3": study_c3, "c5": study_c5, "collision": study_collision,
           "drag_window": study_drag_window}
