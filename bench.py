"""Benchmark: particle-substeps/s of the XPBD substep on one GB300.

Contract line (default): the mixed particles-and-rigid-bodies workload —
1,048,576 particles (128x128x64 lattice, r = 0.005 m, seeded jitter) on the
ground plane and a 256x256-vertex sum-of-sines heightfield (130,050
triangles), plus 1,024 dynamic boxes (half-extents U[0.02, 0.08] m, density
1000 kg/m^3, orientations uniform on SO(3)) dropped onto the pile; plane,
heightfield, moving-box and particle-particle contacts, body contact solve and
body delta apply, dt = 1/60 s, 10 substeps, 1 solver iteration, FP32. One step
= one frame (10 substeps) of one continuous run: the scene is pre-rolled for
--preroll frames (boxes landing in the pile), then --warmup frames, then
--steps timed frames. L2 is flushed (256 MiB write on the solver's stream)
between timed frames; frame times are CUDA events on the solver's stream.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--preroll P] [--impl reference]

The same line carries the other workloads under their own keys:
"particles_on_mesh" (262,144 particles on the heightfield), "pile_1m" (the
plain step at 1,048,576 particles), "batched" (512 uneven scenes in one
batched solver against one solver per scene and against the plain 1M step),
"diff" (forward + backward of the 32,768-particle throw over 600 substeps);
the last key, "headline", repeats each workload's figure.

--impl reference times the CPU restatement of the reference's shaders (the
oracle, all host threads; no product library is loaded) on the same mixed
workload, one substep per step. Under torchrun every rank steps its own
replica of the scene (the path does not shard); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "newton-xpbd-vulkan_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "particle-substeps/s on 1 GB300, plain vs batched graph; fwd+bwd vs fwd time"
UNIT = "particle-substeps/s"
DT = 1.0 / 60.0
SUBSTEPS = 10
ITERATIONS = 1
FLUSH_BYTES = 256 << 20

# Algorithmic bytes per particle for one launch of each kernel (xyz vectors count
# 12 B, scalars 4 B; neighbour gathers, contacts, BVH nodes and the cell table
# count 0 — they can stay cache-resident). The whole substep's compulsory
# traffic is 76 B per particle-substep at one iteration.
ALG_BYTES = {
    "1. Contact Gen (plane + mesh)": 24,       # x, r, flags in; contact header out
    "1d. Contacts on Moving Meshes": 24,       # x, r, flags in; contact header out
    "1b. Contact Ranks (cap)": 12,             # header in; rank out
    "1f. Body Delta Entries (scan, sort)": 4,  # header in
    "2b. Integrate + Cell Keys": 44,           # x, v, w, flags in; key out (+ r in, header out: plane only)
    "2e. Onesweep Pass 0": 12,                 # key in; key, id out
    "2e. Onesweep Pass 1": 16,                 # key, id in and out
    "2e. Onesweep Pass 2": 16,
    "2e. Onesweep Pass 3": 16,
    "2g. Cell Table + Gather": 88,             # sorted key, id, x, v, w, r, flags in; 36 B of records out
    "3. Solve+Apply(+Restitution)": 96,        # records, id, x0, v0, header in; x, v out
    "3c. Restitution (bodies)": 52,            # header, x0, v0, v in; v out
}
STEP_ALG_BYTES = 76
SLOT_BYTES = 48  # one contact slot (body point, normal, body velocity: 3 float4) read by the solve


def alg_bytes(stage, n, contacts=0):
    """Algorithmic bytes of one launch of a stage over n particles; the solve also reads the
    substep's contact slots (contacts = the contact count of a substep)."""
    extra = SLOT_BYTES * contacts if stage.startswith("3. Solve") else 0
    return ALG_BYTES[stage] * n + extra


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def reduce_max(value: float, world: int) -> float:
    """Max over ranks (identity for one rank)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def make_solver(sc, device_index=-1):
    """A vkxpbd solver holding scene `sc` (meshes, bodies, particles)."""
    import vkxpbd

    cfg = vkxpbd.SolverConfig()
    sc.apply_config(cfg)
    cfg.device_index = device_index
    s = vkxpbd.XpbdSolver()
    s.init(cfg, sc.n)
    for (v, t, margin, wt) in sc.meshes:
        s.add_mesh(v, t, shape_margin=margin, is_watertight=wt)
    s.finalize_meshes()
    b = getattr(sc, "bodies", None)
    if b is not None:
        s.set_bodies(b.q, b.qd, b.com, b.inertia, b.inv_inertia, b.inv_mass, b.flags)
    s.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
    return s, cfg


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for name, val in zip(names, f[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def dram_traffic(workload: str, kernel_stage: str):
    """Per-launch DRAM bytes of a kernel at this workload from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as fh:
            entry = json.load(fh).get(workload, {})
        return entry.get(kernel_stage) if isinstance(entry, dict) else None
    except (OSError, ValueError):
        return None


def launches_of(stage, prof_substeps):
    per_iteration = stage.startswith(("3.", "3b", "3d"))
    return prof_substeps * (ITERATIONS if per_iteration else 1)


def stage_table(stage_ms, prof_substeps, n, peak, contacts=0):
    out = {}
    for k, v in stage_ms.items():
        if v <= 0:
            continue
        us = v / launches_of(k, prof_substeps) * 1e3
        st = {"us_per_launch": round(us, 2)}
        if k in ALG_BYTES:
            gbs = alg_bytes(k, n, contacts) / (us * 1e-6) / 1e9
            st.update({"achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)})
        out[k] = st
    return out


def profile_stages(solver, frames, flush=None):
    """Per-kernel device times from event-record nodes inside the frame graph (a separate,
    serialised pass: the timed frames run two streams)."""
    solver.set_profiling(True)
    solver.reset_stage_times()
    for _ in range(frames):
        if flush is not None:
            flush()
        solver.step(DT, SUBSTEPS, ITERATIONS)
    stage_ms, prof_substeps = solver.get_stage_times()
    solver.set_profiling(False)
    return stage_ms, prof_substeps


def roofline_of(workload, stage_ms, prof_substeps, n, step_ms, peak, peak_kind, contacts=0):
    """Dominant kernel (most device time among the kernels with algorithmic bytes) against
    the measured HBM copy bandwidth, and the whole substep with 76 B per particle-substep.
    contacts: a substep's contact count (the solve reads one 48-byte slot per contact)."""
    ranked = sorted(((v, k) for k, v in stage_ms.items() if k in ALG_BYTES and v > 0), reverse=True)
    if not ranked:
        raise RuntimeError(f"no per-kernel stage times were recorded: {stage_ms}")
    dom_ms, dom = ranked[0]
    avg_ms = dom_ms / launches_of(dom, prof_substeps)
    achieved = alg_bytes(dom, n, contacts) / (avg_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "alg_bytes_per_launch": alg_bytes(dom, n, contacts), "avg_launch_us": round(avg_ms * 1e3, 2),
                "traffic": dram_traffic(workload, dom),
                "share_of_step": round(dom_ms / sum(v for v in stage_ms.values() if v > 0), 3)}
    step_gbs = STEP_ALG_BYTES * n * SUBSTEPS * ITERATIONS / (step_ms * 1e-3) / 1e9
    roofline_step = {"alg_bytes_per_particle_substep": STEP_ALG_BYTES, "achieved": round(step_gbs, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(step_gbs / peak, 4), "peak_source": peak_kind}
    return roofline, roofline_step


def timed_frames(solver, stream, frames, flush=None, per_frame=False):
    """Device time (ms) of `frames` frames, CUDA events on the solver's stream. per_frame:
    also each frame's device time and kernel count (the kernels of the graph it replayed)."""
    import torch

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(frames)]
    kernels = []
    for k in range(frames):
        # the previous frame is finished (its status read back) before this one is queued, so
        # the launch below waits for nothing; the flush then runs on the device while the host
        # launches the frame, and the host's turnaround stays outside the frame's events
        solver.sync()
        if flush is not None:
            flush()
        ev[k][0].record(stream)
        before = solver.kernels_launched if per_frame else 0
        solver.step_async(DT, SUBSTEPS, ITERATIONS)
        ev[k][1].record(stream)
        if per_frame:
            kernels.append(solver.kernels_launched - before)
    solver.sync()
    torch.cuda.synchronize()
    times = [a.elapsed_time(b) for a, b in ev]
    return (sum(times), times, kernels) if per_frame else sum(times)


def e2e_frames(solver, frames, x, v, body_q=None, body_qd=None, flush=None, sync=None):
    """The same frames through the public API with host buffers: every frame uploads the state
    (set_particles, and set_bodies for bodies), steps, and reads the state back. Returns
    (seconds, h2d bytes per frame, d2h bytes per frame)."""
    x_h, v_h = x.copy(), v.copy()
    q_h = None if body_q is None else body_q.copy()
    qd_h = None if body_qd is None else body_qd.copy()
    nbytes = x_h.nbytes + v_h.nbytes + (0 if q_h is None else q_h.nbytes + qd_h.nbytes)
    total = 0.0
    for _ in range(frames):
        if flush is not None:
            flush()
        if sync is not None:
            sync()
        t0 = time.perf_counter()
        solver.set_particles(x_h, v_h)
        if q_h is not None:
            solver.set_bodies(q_h, qd_h)
        solver.step(DT, SUBSTEPS, ITERATIONS)
        x_h = solver.get_positions()
        v_h = solver.get_velocities()
        if q_h is not None:
            q_h = solver.get_body_q()
            qd_h = solver.get_body_qd()
        total += time.perf_counter() - t0
    return total, nbytes, nbytes


def cpu_baseline_sample(sc, x, v, body_q=None, body_qd=None, budget_s=15.0):
    """Oracle (CPU restatement, all host threads) on the pre-rolled state: a bounded number of
    substeps of the same workload."""
    import oracle as O
    from helpers import config_for, make_pair

    O.load("f32").or_set_threads(os.cpu_count() or 1)
    cfg = config_for(sc, gpu=False)
    _, orc = make_pair(sc, cfg, gpu=False)
    orc.set_particles(x, v)
    if body_q is not None:
        orc.set_bodies(body_q, body_qd)
    sdt = DT / SUBSTEPS
    t0 = time.perf_counter()
    orc.step(sdt, 1, ITERATIONS)
    t1 = time.perf_counter() - t0
    more = max(0, min(10 * SUBSTEPS, int(budget_s / max(t1, 1e-3)) - 1))
    t0 = time.perf_counter()
    for _ in range(more):
        orc.step(sdt, 1, ITERATIONS)
    t2 = time.perf_counter() - t0
    total_t, total_sub = t1 + t2, 1 + more
    return {"value": sc.n * total_sub / total_t, "unit": UNIT, "cores": int(O.load("f32").or_get_threads()),
            "kind": "port",
            "sample": f"{total_sub} substeps (dt/10 each) of the pre-rolled {sc.n}-particle {sc.name} state "
                      f"({total_t:.1f} s)"}


def finite(obj):
    """The result with every non-finite float replaced by None (valid JSON)."""
    if isinstance(obj, dict):
        return {k: finite(v) for k, v in obj.items()}
    if isinstance(obj, (list, tuple)):
        return [finite(v) for v in obj]
    if isinstance(obj, float) and not np.isfinite(obj):
        return None
    return obj


def headline(result):
    """Each workload's figure, repeated compactly at the end of the line."""
    head = {"mixed": result["value"], "mixed_e2e": result["e2e"]["value"],
            "mixed_roofline_frac": result["roofline"]["frac"]}
    pom = result.get("particles_on_mesh", {})
    if "value" in pom:
        head["particles_on_mesh"] = pom["value"]
        head["particles_on_mesh_e2e"] = pom["e2e"]["value"]
    pile = result.get("pile_1m", {})
    if "value" in pile:
        head["pile_1m"] = pile["value"]
        head["pile_1m_roofline_step_frac"] = pile["roofline_step"]["frac"]
    bat = result.get("batched", {})
    for k, name in (("batched_value", "batched"), ("plain_value", "batched_plain"),
                    ("batched_over_plain", "batched_over_plain"), ("batched_over_pile_1m", "batched_over_pile_1m")):
        if k in bat:
            head[name] = bat[k]
    diff = result.get("diff", {})
    for k in ("fwd_bwd_over_fwd", "forward_value"):
        if k in diff:
            head["diff_" + k] = diff[k]
    if "grad_checked" in diff:
        head["diff_grad_mu_60_substeps"] = diff["grad_checked"]["soft_contact_mu"]
    if "cpu_baseline" in result:
        head["cpu_baseline"] = result["cpu_baseline"]["value"]
    small = result.get("pile_4k", {})
    if "value" in small:
        head["pile_4k"] = small["value"]
    for name in ("pile_4k", "particles_on_mesh", "batched"):
        cpu = (result.get(name) or {}).get("cpu_baseline")
        if cpu:
            head[name + "_cpu"] = cpu["value"]
    return head


def run_gpu(args):
    import torch

    import scenes

    rank, world, local = dist_env()
    if args.only and "main" not in args.only.split(","):  # sub-measurements alone (not the contract line)
        dev = torch.device("cuda", local)
        parts = {}
        for key, name, fn in (("mesh", "particles_on_mesh", measure_mesh), ("batched", "batched", measure_batched),
                              ("diff", "diff", measure_diff), ("pile", "pile_1m", measure_pile),
                              ("pile4k", "pile_4k", measure_small_pile)):
            if key in args.only.split(","):
                parts[name] = fn(args, dev)
        print(json.dumps(parts), flush=True)
        return
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    dev = torch.device("cuda", local)
    sc = scenes.mixed()
    solver, _ = make_solver(sc, device_index=local)
    if args.load_state:  # a pre-rolled state saved by --save-state (short profiling runs)
        st = np.load(args.load_state)
        solver.set_particles(st["x"], st["v"])
        solver.set_bodies(st["q"], st["qd"])
    else:
        for _ in range(args.preroll):
            solver.step(DT, SUBSTEPS, ITERATIONS)
    x_snap, v_snap = solver.get_positions(), solver.get_velocities()
    q_snap, qd_snap = solver.get_body_q(), solver.get_body_qd()
    if args.save_state:
        np.savez(args.save_state, x=x_snap, v=v_snap, q=q_snap, qd=qd_snap)

    stream = torch.cuda.ExternalStream(solver.cuda_stream, device=dev)
    flush_buf = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def flush():
        with torch.cuda.stream(stream):
            flush_buf.fill_(1.0)

    for _ in range(args.warmup):
        flush()
        solver.step(DT, SUBSTEPS, ITERATIONS)
    # the timed frames start here; the end-to-end pass below steps the same frames again
    x_t0, v_t0 = solver.get_positions(), solver.get_velocities()
    q_t0, qd_t0 = solver.get_body_q(), solver.get_body_qd()
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize(dev)
    kernels_before = solver.kernels_launched
    if args.profile_timed:  # a profiler started with collection off (ncu --profile-from-start off) sees these frames
        torch.cuda.profiler.start()
    dev_ms, frame_ms, frame_kernels = timed_frames(solver, stream, args.steps, flush, per_frame=True)
    choices = {"solve_form": solver.solve_form, "solve_split": solver.solve_split}
    if args.profile_timed:
        torch.cuda.synchronize(dev)
        torch.cuda.profiler.stop()
    kernels_timed = solver.kernels_launched - kernels_before
    torch.cuda.synchronize(dev)
    barrier(world)
    clk = clocks.stop()
    dev_ms_max = reduce_max(dev_ms, world)
    particle_substeps = sc.n * SUBSTEPS * args.steps * world
    value = particle_substeps / (dev_ms_max * 1e-3)

    stage_ms, prof_substeps = profile_stages(solver, min(args.steps, 10), flush)
    peak, peak_kind = measured_peak_hbm()
    contacts = int(solver.last_contact_count)  # the last profiled substep's
    roofline, roofline_step = roofline_of("mixed", stage_ms, prof_substeps, sc.n, dev_ms / args.steps, peak,
                                          peak_kind, contacts)

    # end to end through the public API with host buffers: set_particles + set_bodies -> step -> readback,
    # from the state the timed frames started from, so both cover the same frames
    e2e_s, h2d, d2h = e2e_frames(solver, args.steps, x_t0, v_t0, q_t0, qd_t0, flush,
                                 lambda: torch.cuda.synchronize(dev))
    e2e_s = reduce_max(e2e_s, world)
    e2e = {"value": particle_substeps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h)}
    bq, bqd = solver.get_body_q()[1:], solver.get_body_qd()[1:]

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded lattice, sum-of-sines heightfield, seeded boxes)",
        "config": {"workload": "mixed", "particles": sc.n, "boxes": len(sc.meshes) - 1,
                   "triangles": int(sum(m[1].shape[0] for m in sc.meshes)),
                   "substeps": SUBSTEPS, "iterations": ITERATIONS, "dt": DT, "step": "one frame (10 substeps)",
                   "preroll_frames": args.preroll, "l2": "flushed between steps (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "roofline": roofline,
        "roofline_step": roofline_step,
        "stages": stage_table(stage_ms, prof_substeps, sc.n, peak, contacts),
        "contacts_last_substep": contacts,
        "boxes_finite": bool(np.isfinite(bq).all() and np.isfinite(bqd).all()),
        "e2e": e2e, "gpu_launches": int(kernels_timed), "clocks": clk,
        # each timed frame's device time and kernel count (a frame whose first iteration is
        # split launches one solve kernel more per substep), and the solver's choices after them
        "frames": {"ms": [round(t, 3) for t in frame_ms], "kernels": [int(c) for c in frame_kernels],
                   "choices_after": choices},
    }
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline_sample(sc, x_snap, v_snap, q_snap, qd_snap, budget_s=args.cpu_budget)
    del solver
    for name, on, fn in (("pile_4k", args.small_pile, lambda: measure_small_pile(args, dev)),
                         ("particles_on_mesh", args.mesh_frames > 0, lambda: measure_mesh(args, dev)),
                         ("pile_1m", args.pile_frames > 0, lambda: measure_pile(args, dev)),
                         ("batched", args.batched_scenes > 0, lambda: measure_batched(args, dev)),
                         ("diff", args.diff_frames > 0, lambda: measure_diff(args, dev))):
        if rank == 0 and on:
            try:
                result[name] = fn()
            except RuntimeError as e:  # a device-side table overflow is reported, not fatal to the line
                result[name] = {"error": str(e)}
    if rank == 0:
        pile = result.get("pile_1m", {}).get("value")
        bat = result.get("batched", {})
        if pile and bat.get("batched_value"):
            bat["batched_over_pile_1m"] = bat["batched_value"] / pile
        result["headline"] = headline(result)
        print(json.dumps(finite(result)), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def measure_mesh(args, dev):
    """Particles on a mesh: 262,144 particles (64^3 lattice, r 0.005, seed 42) falling onto the
    256x256 sum-of-sines heightfield (130,050 triangles, seed 44) with plane, mesh and
    particle-particle contacts, 10 substeps x 1 iteration per frame, device-timed frames after
    a pre-roll (the pile is in contact), L2 flushed between frames; plus the same frames end
    to end through the public API with host buffers, and the frame cache."""
    import torch

    import scenes

    sc = scenes.particles_on_mesh()
    s, _ = make_solver(sc, device_index=dev.index)
    for _ in range(args.mesh_preroll):
        s.step(DT, SUBSTEPS, ITERATIONS)
    x_snap, v_snap = s.get_positions(), s.get_velocities()
    stream = torch.cuda.ExternalStream(s.cuda_stream, device=dev)
    flush_buf = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def flush():
        with torch.cuda.stream(stream):
            flush_buf.fill_(1.0)

    for _ in range(args.warmup):
        flush()
        s.step(DT, SUBSTEPS, ITERATIONS)
    x_t0, v_t0 = s.get_positions(), s.get_velocities()  # where the timed frames (and the e2e pass) start
    frames = args.mesh_frames
    torch.cuda.synchronize(dev)
    dev_ms = timed_frames(s, stream, frames, flush)
    stage_ms, prof_substeps = profile_stages(s, min(frames, 30), flush)
    peak, peak_kind = measured_peak_hbm()
    contacts = int(s.last_contact_count)
    roofline, roofline_step = roofline_of("particles_on_mesh", stage_ms, prof_substeps, sc.n, dev_ms / frames,
                                          peak, peak_kind, contacts)
    e2e_s, h2d, d2h = e2e_frames(s, frames, x_t0, v_t0, flush=flush, sync=lambda: torch.cuda.synchronize(dev))
    work = sc.n * SUBSTEPS * frames
    out = {"workload": "particles_on_mesh", "particles": sc.n, "triangles": int(sc.meshes[0][1].shape[0]),
           "preroll_frames": args.mesh_preroll, "frames": frames, "value": work / (dev_ms * 1e-3), "unit": UNIT,
           "ms_per_frame": dev_ms / frames, "roofline": roofline, "roofline_step": roofline_step,
           "stages": stage_table(stage_ms, prof_substeps, sc.n, peak, contacts),
           "e2e": {"value": work / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                   "d2h_bytes_per_step": int(d2h)}}
    if args.cache_frames > 0:
        out["frame_cache"] = measure_cache(args, s, sc)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_sample(sc, x_snap, v_snap, budget_s=args.cpu_budget / 3)
    return out


def measure_small_pile(args, dev):
    """The reference's own CPU-runnable case: the 4,096-particle pile (16^3 lattice, r 0.01 m,
    spacing 0.02 m, jitter +/-0.002 m, seed 42, plane + particle contacts), 120 frames of 10
    substeps from the initial state, on the GPU (device-timed, one graph per frame; at this
    size the step is launch-bound) and on the oracle (all host threads)."""
    import torch

    import oracle as O
    import scenes
    from helpers import config_for, make_pair

    sc = scenes.pile()
    frames = 120
    s, _ = make_solver(sc, device_index=dev.index)
    for _ in range(args.warmup):  # graph capture and sort tuning, then back to the initial state
        s.step(DT, SUBSTEPS, ITERATIONS)
    s.set_particles(sc.positions, sc.velocities)
    stream = torch.cuda.ExternalStream(s.cuda_stream, device=dev)
    torch.cuda.synchronize(dev)
    dev_s = timed_frames(s, stream, frames) * 1e-3
    work = sc.n * SUBSTEPS * frames
    out = {"workload": "pile_4k", "particles": sc.n, "frames": frames, "value": work / dev_s, "unit": UNIT,
           "ms_per_frame": dev_s / frames * 1e3}
    if not args.no_cpu_baseline:
        O.load("f32").or_set_threads(os.cpu_count() or 1)
        _, orc = make_pair(sc, config_for(sc, gpu=False), gpu=False)
        t0 = time.perf_counter()
        done = 0
        while done < frames and time.perf_counter() - t0 < args.cpu_budget / 3:
            orc.step(DT, SUBSTEPS, ITERATIONS)
            done += 1
        t = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sc.n * SUBSTEPS * done / t, "unit": UNIT,
                               "cores": int(O.load("f32").or_get_threads()), "kind": "port",
                               "sample": f"{done} frames of 10 substeps from the initial state ({t:.1f} s)"}
    return out


def measure_batched(args, dev):
    """Batched uneven scenes: 512 piles with log-uniform counts in [1024, 65536] (seed 46),
    each with 0..16 dynamic boxes (--batched-boxes; half-extents U[0.02, 0.08], seed 46 + s)
    dropped onto it, plane + particle-particle + box contacts, 10 substeps x 1 iteration per
    frame. "batched" is one solver stepping all scenes (one graph per frame, one launch per
    kernel for all scenes, every box assigned to its scene); "plain" is one solver per scene,
    each frame stepped scene by scene with the blocking step(), as a reference user drives
    several scenes. Aggregate particle-substeps/s."""
    import torch
    import vkxpbd

    import scenes

    if args.batched_boxes > 0:
        batch = scenes.batched_piles_with_boxes(args.batched_scenes, max_boxes=args.batched_boxes)
    else:
        batch = scenes.batched_piles(args.batched_scenes)
    cfg = vkxpbd.SolverConfig()
    batch.apply_config(cfg)
    cfg.device_index = dev.index
    g = vkxpbd.XpbdSolver()
    g.init_batched(cfg, batch.counts)

    def add_bodies(solver, meshes, bodies, body_scene=None):
        for (v, t, margin, wt) in meshes:
            solver.add_mesh(v, t, shape_margin=margin, is_watertight=wt)
        solver.finalize_meshes()
        if bodies is not None:
            solver.set_bodies(bodies.q, bodies.qd, bodies.com, bodies.inertia, bodies.inv_inertia,
                              bodies.inv_mass, bodies.flags)
            if body_scene is not None:
                solver.set_body_scenes(body_scene)

    n_boxes = 0
    if args.batched_boxes > 0:
        meshes, bodies, body_scene = scenes.batch_bodies(batch)
        add_bodies(g, meshes, bodies, body_scene)
        n_boxes = int((body_scene >= 0).sum())
    else:
        g.finalize_meshes()
    g.set_particles(batch.concat("positions"), batch.concat("velocities"), batch.concat("inv_mass"),
                    batch.concat("radii"), batch.concat("flags"))
    frames = args.batched_frames
    stream = torch.cuda.ExternalStream(g.cuda_stream, device=dev)
    for _ in range(args.warmup):
        g.step(DT, SUBSTEPS, ITERATIONS)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    dev_b = timed_frames(g, stream, frames) * 1e-3
    wall_b = time.perf_counter() - t0
    launches_b = g.get_frame_stats()["kernels_per_frame"]
    work = batch.n * SUBSTEPS * frames
    stage_ms, prof_substeps = profile_stages(g, min(frames, 5))
    peak, peak_kind = measured_peak_hbm()
    step_gbs = STEP_ALG_BYTES * work / dev_b / 1e9
    del g
    torch.cuda.synchronize(dev)

    plain = []
    for sc in batch.scenes:
        s = vkxpbd.XpbdSolver()
        s.init(cfg, sc.n)
        add_bodies(s, sc.meshes, sc.bodies)
        s.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
        plain.append(s)
    for _ in range(args.warmup):
        for s in plain:
            s.step(DT, SUBSTEPS, ITERATIONS)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(frames):
        for s in plain:
            s.step(DT, SUBSTEPS, ITERATIONS)
    torch.cuda.synchronize(dev)
    wall_p = time.perf_counter() - t0
    launches_p = sum(s.get_frame_stats()["kernels_per_frame"] for s in plain)
    del plain
    cpu = None
    if not args.no_cpu_baseline:  # the oracle stepping every 32nd scene in turn, one frame each
        import oracle as O
        from helpers import config_for, make_pair

        O.load("f32").or_set_threads(os.cpu_count() or 1)
        sample = batch.scenes[::32]
        orcs = [make_pair(sc, config_for(sc, gpu=False), gpu=False)[1] for sc in sample]
        t0 = time.perf_counter()
        for orc in orcs:
            orc.step(DT, SUBSTEPS, ITERATIONS)
        t = time.perf_counter() - t0
        n_s = sum(sc.n for sc in sample)
        cpu = {"value": n_s * SUBSTEPS / t, "unit": UNIT, "cores": int(O.load("f32").or_get_threads()),
               "kind": "port", "sample": f"one frame of every 32nd scene ({len(sample)} scenes, {n_s} particles, "
                                         f"their boxes) stepped one scene after another ({t:.1f} s)"}
    return {"workload": "batched_piles", "scenes": len(batch.scenes), "particles": batch.n, "boxes": n_boxes,
            "counts": "log-uniform 1024-65536, seed 46", "frames": frames, "warmup": args.warmup,
            "batched_value": work / dev_b, "batched_wall_value": work / wall_b, "plain_value": work / wall_p,
            "unit": UNIT, "batched_over_plain": (work / wall_b) / (work / wall_p),
            "launches_per_frame": {"batched": int(launches_b), "plain": int(launches_p)},
            "roofline_step": {"alg_bytes_per_particle_substep": STEP_ALG_BYTES, "achieved": round(step_gbs, 1),
                              "peak": peak, "unit": "GB/s", "frac": round(step_gbs / peak, 4),
                              "peak_source": peak_kind},
            "stages": stage_table(stage_ms, prof_substeps, batch.n, peak),
            "cpu_baseline": cpu,
            "note": "batched_value device-timed (CUDA events); *_wall_value and plain_value host wall clock "
                    "around stepping; batched_over_pile_1m = batched_value / the pile_1m value"}


def measure_pile(args, dev):
    """Plain step at 1M particles: the 4,096-particle pile recipe (r 0.01 m, spacing 0.02 m,
    jitter +/-0.002 m, seed 42, plane + particle contacts, cell 0.02 m) on a 128x128x64
    lattice (1,048,576 particles), 10 substeps x 1 iteration per frame, device-timed frames
    after a pre-roll (the lattice has settled into contact). Reported beside the HBM roofline
    of the whole substep (76 B per particle-substep)."""
    import torch

    import scenes

    sc = scenes.pile(dims=(128, 128, 64), name="pile_1m")
    s, _ = make_solver(sc, device_index=dev.index)
    if args.pile_solve_form >= 0:  # a fixed solve-kernel form instead of the solver's timed choice
        s.set_solve_form(args.pile_solve_form)
    for _ in range(args.pile_preroll + args.warmup):
        s.step(DT, SUBSTEPS, ITERATIONS)
    stream = torch.cuda.ExternalStream(s.cuda_stream, device=dev)
    frames = args.pile_frames
    torch.cuda.synchronize(dev)
    dev_s = timed_frames(s, stream, frames) * 1e-3
    launches = s.get_frame_stats()["kernels_per_frame"]
    stage_ms, prof_substeps = profile_stages(s, min(frames, 5))
    peak, peak_kind = measured_peak_hbm()
    work = sc.n * SUBSTEPS * frames
    contacts = int(s.last_contact_count)
    roofline, roofline_step = roofline_of("pile_1m", stage_ms, prof_substeps, sc.n, dev_s * 1e3 / frames, peak,
                                          peak_kind, contacts)
    return {"workload": "pile_1m", "particles": sc.n, "preroll_frames": args.pile_preroll, "frames": frames,
            "value": work / dev_s, "unit": UNIT, "ms_per_frame": dev_s / frames * 1e3,
            "launches_per_frame": int(launches), "contacts_last_substep": int(s.last_contact_count),
            "roofline": roofline, "roofline_step": roofline_step,
            "stages": stage_table(stage_ms, prof_substeps, sc.n, peak, contacts)}


def measure_cache(args, solver, sc):
    """The add-on's per-frame cache (step, then np.save of the positions): done synchronously
    as the add-on does, and with the frame recorder (copy + file write overlap the next frame)."""
    import tempfile

    frames = args.cache_frames
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        for f in range(frames):
            solver.step(DT, SUBSTEPS, ITERATIONS)
            np.save(os.path.join(d, f"frame_{f + 1:04d}.npy"), solver.get_positions())
        sync_s = time.perf_counter() - t0
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        solver.record_start(d, 1)
        for f in range(frames):
            solver.step_async(DT, SUBSTEPS, ITERATIONS)
        written = solver.record_stop()
        rec_s = time.perf_counter() - t0
    work = sc.n * SUBSTEPS * frames
    return {"frames": frames, "bytes_per_frame": sc.n * 12, "files_written": written, "unit": UNIT,
            "synchronous_value": work / sync_s, "recorder_value": work / rec_s,
            "note": "host wall clock; synchronous = step + get_positions + np.save per frame"}


def measure_diff(args, dev):
    """Differentiable throw: 32,768 particles (32^3, spacing 0.02, r 0.01) with velocities
    N((2,3,0), 0.1^2) (seed 43), 600 substeps (60 frames x 10), plane + particle contacts,
    checkpoint every 20 substeps; loss = |mean(x_final) - target|^2 (target seed 47).
    Forward = the checkpointed rollout; backward = replay + adjoint of every substep."""
    import torch
    import vkxpbd

    import scenes

    sc = scenes.throw()
    target = scenes.throw_target()
    cfg = vkxpbd.SolverConfig()
    sc.apply_config(cfg)
    cfg.device_index = dev.index
    s = vkxpbd.XpbdSolver()
    s.init(cfg, sc.n)
    s.finalize_meshes()
    frames, ckpt = args.diff_frames, 2
    fwd, bwd = [], []
    for rep in range(args.diff_reps + 1):  # first repetition warms up (graph capture, allocations)
        s.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        s.rollout(DT, SUBSTEPS, frames, 1, ckpt)
        x = s.get_positions()
        t1 = time.perf_counter()
        m = x.astype(np.float64).mean(axis=0)
        gx = np.tile((2.0 * (m - target) / sc.n).astype(np.float32), (sc.n, 1))
        t2 = time.perf_counter()
        g = s.rollout_backward(gx)
        t3 = time.perf_counter()
        if rep:
            fwd.append(t1 - t0)
            bwd.append(t3 - t2)
    f, b = statistics.median(fwd), statistics.median(bwd)
    # growth of the exact gradient with the horizon (the Jacobian of the contact projection
    # in a dense pile has modes larger than 1 per substep)
    growth = {}
    for hf in (1, 3, 6, 7, 12, 24):
        s.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
        s.rollout(DT, SUBSTEPS, hf, 1, ckpt)
        mh = s.get_positions().astype(np.float64).mean(axis=0)
        gh = s.rollout_backward(np.tile((2.0 * (mh - target) / sc.n).astype(np.float32), (sc.n, 1)))
        growth[str(hf * SUBSTEPS)] = {"v0_norm": float(np.linalg.norm(gh["v0"])),
                                      "v0_sum": [float(a) for a in gh["v0"].astype(np.float64).sum(axis=0)],
                                      "soft_contact_mu": float(gh["soft_contact_mu"]),
                                      "soft_contact_restitution": float(gh["soft_contact_restitution"])}
    return {"workload": "diff_throw", "particles": sc.n, "substeps": frames * SUBSTEPS,
            "checkpoint_substeps": ckpt * SUBSTEPS, "reps": args.diff_reps, "forward_s": f, "backward_s": b,
            "fwd_bwd_over_fwd": (f + b) / f, "forward_value": sc.n * frames * SUBSTEPS / f, "unit": UNIT,
            "loss": float(((m - target) ** 2).sum()),
            "grad": {"soft_contact_mu": g["soft_contact_mu"], "particle_mu": g["particle_mu"],
                     "soft_contact_restitution": g["soft_contact_restitution"],
                     "v0_norm": float(np.linalg.norm(g["v0"])), "inv_mass_norm": float(np.linalg.norm(g["inv_mass"]))},
            "gradient_vs_horizon_substeps": growth,
            "grad_checked": dict(growth["60"], horizon_substeps=60,
                                 check="central differences (eps 1e-3) of the FP64 oracle forward; plane friction "
                                       "and uniform velocity shifts within 1e-3 relative (GPU test)"),
            "note": "host wall clock around xpbd_rollout / xpbd_rollout_backward (synchronous calls); past ~80 "
                    "substeps the exact gradient grows exponentially (FP64 as FP32), non-finite values print as "
                    "null"}


def run_reference(args):
    """The reference's CPU implementation of the path: the oracle port (a restatement of the
    reference's shaders and host driver) on all host threads, on the mixed workload. Loads no
    product library: the scene comes from the seeded generators and the configuration from
    the oracle's own SolverConfig (the reference's defaults, src/scene.h:15-40)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle as O
    from helpers import config_for, make_pair

    import scenes

    O.load("f32").or_set_threads(os.cpu_count() or 1)
    sc = scenes.mixed()
    cfg = config_for(sc, gpu=False)
    _, orc = make_pair(sc, cfg, gpu=False)
    for _ in range(args.ref_preroll):
        orc.step(DT, SUBSTEPS, ITERATIONS)
    sdt = DT / SUBSTEPS  # one step = one substep of the frame (dt/10)
    for _ in range(args.warmup):
        orc.step(sdt, 1, ITERATIONS)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.step(sdt, 1, ITERATIONS)
    t = time.perf_counter() - t0
    value = sc.n * args.steps / t
    cores = int(O.load("f32").or_get_threads())
    sample = (f"{args.steps} substeps (dt/10 each) of the mixed workload after {args.ref_preroll} pre-roll frames "
              f"and {args.warmup} warm-up substeps; like the reference's shader, the oracle queries every particle "
              f"against every mesh, a cost that does not depend on the pile's state")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded lattice, sum-of-sines heightfield, seeded boxes)",
           "config": {"workload": "mixed", "particles": sc.n, "boxes": len(sc.meshes) - 1,
                      "triangles": int(sum(m[1].shape[0] for m in sc.meshes)), "substeps": SUBSTEPS,
                      "iterations": ITERATIONS, "dt": DT, "step": "one substep (dt/10)",
                      "preroll_frames": args.ref_preroll, "parallelism": "cpu threads"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--preroll", type=int, default=20, help="mixed workload frames before the timed frames")
    ap.add_argument("--ref-preroll", type=int, default=0, help="reference arm: oracle frames before timing")
    ap.add_argument("--save-state", default="", help="save the mixed workload's pre-rolled state (.npz)")
    ap.add_argument("--load-state", default="", help="start the mixed workload from a saved state (no pre-roll)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mesh-frames", type=int, default=100, help="0 skips the particles-on-mesh measurement")
    ap.add_argument("--mesh-preroll", type=int, default=30)
    ap.add_argument("--batched-scenes", type=int, default=512, help="0 skips the batched-scenes measurement")
    ap.add_argument("--batched-frames", type=int, default=10)
    ap.add_argument("--batched-boxes", type=int, default=16, help="0..N dynamic boxes per batched scene (0: none)")
    ap.add_argument("--diff-frames", type=int, default=60, help="0 skips the differentiable rollout measurement")
    ap.add_argument("--cache-frames", type=int, default=50, help="0 skips the frame-cache measurement")
    ap.add_argument("--diff-reps", type=int, default=3)
    ap.add_argument("--pile-frames", type=int, default=10, help="0 skips the 1M-particle plain pile measurement")
    ap.add_argument("--no-small-pile", dest="small_pile", action="store_false",
                    help="skip the 4,096-particle pile (the reference's CPU-runnable case)")
    ap.add_argument("--pile-preroll", type=int, default=20)
    ap.add_argument("--pile-solve-form", type=int, default=-1, help="fix the 1M pile's solve form (-1: timed choice)")
    ap.add_argument("--profile-timed", action="store_true",
                    help="bracket the mixed workload's timed frames with cudaProfilerStart/Stop")
    ap.add_argument("--only", default="", help="comma list of parts to run alone: mesh,batched,diff,pile,pile4k")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
