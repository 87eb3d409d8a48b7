#!/usr/bin/env python3
"""Benchmark of the kazan GB300 draw path.

Workload (default): the batched command buffer - 4,096 vkCmdDrawIndexed draws (log-uniform triangle
counts in [16, 65536], each its own sphere mesh and MVP push constant, Lambert VS/FS) into a 2048x2048
RGBA8 + D32 target, seeded synthetic scene (seed 3).  One step = one vkQueueSubmit of the recorded command
buffer (--mode batched: one launch per pipeline phase), i.e. one full render of the scene.  `value` times
K submissions of the command buffer as an application records it (a CUDA graph whose kernels are chained
by programmatic dependent launch).  The same K submissions are then timed again from a second recording
of the same draws with the driver's kernel timing on, where every kernel launch is bracketed by CUDA
events on the queue stream: the `kernels` table and the roofline (the dominant kernel's mean duration)
come from that pass, `kernel_pass` gives its step time.

Printed JSON line (rank 0):
  value      Mtris/s with vertex/index buffers and attachments resident in HBM (device-local memory),
             K submissions timed with CUDA events on the queue's stream
  e2e        the same metric through host-visible memory: every step uploads the vertex and index buffers
             from pinned host memory, renders, downloads the colour image and reads it on the host
  per_draw   the plain per-draw launch form of the same command buffer (the batching baseline)
  roofline   achieved HBM bandwidth of the dominant kernel (algorithmic bytes / kernel time) vs measured peak
  cpu_baseline  the CPU oracle (project restatement; the reference has no CPU rasteriser) on a bounded
             sample of the draws, all host threads
  persistent the same draws in the persistent schedule (one cooperative kernel per submission)
  autotune   the autotuner's measured candidates and its choice (schedule, tile, visibility-path knobs)
  other_workloads  short timings of the other render configurations (plain small draw, single large draw,
             ordered blend, textured draw) and one rate of the serving loop (p50 / p99 latency)
--impl reference times that CPU path alone (the reference arm).  Under torchrun each rank renders its own
replica (no data-path collective); value = triangles of all ranks / max time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "single", "soup", "blend", "textured", "serve"])
    ap.add_argument("--budget-gb", type=float, default=40.0, help="serve: HBM admission budget")
    ap.add_argument("--ndraws", type=int, default=4096)
    ap.add_argument("--tile", type=int, default=16)
    ap.add_argument("--mode", default="batched", choices=["persistent", "batched", "perdraw"])
    ap.add_argument("--samples", type=int, default=1, choices=[1, 4],
                    help="4: multisampled colour and depth attachments resolved at the end of the pass")
    ap.add_argument("--depth-format", default="d32", choices=["d32", "d16", "d24s8"])
    ap.add_argument("--indirect", default="none", choices=["none", "host", "device"],
                    help="record the draws as vkCmdDraw*Indirect over commands in host-visible memory, or in "
                         "device memory written by a vkCmdCopyBuffer in the same command buffer")
    ap.add_argument("--no-perdraw", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (use --mode / --tile as given)")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the short timings of the other render configurations in the default run")
    return ap.parse_args()


def make_scene(args):
    scene, cfg = _base_scene(args)
    if args.samples != 1 or args.depth_format != "d32":
        import dataclasses
        scene = dataclasses.replace(scene, samples=args.samples, depth_format=args.depth_format)
        cfg = dict(cfg, workload=cfg["workload"] + ", %dx samples, %s depth" % (args.samples, args.depth_format.upper()))
    return scene, cfg


def _base_scene(args):
    from kazan_gb300 import scenes
    if args.workload == "batched":
        return scenes.batched(ndraws=args.ndraws), {"workload": "batched: %d vkCmdDrawIndexed, 2048x2048 RGBA8+D32, "
                                                    "tris/draw log-uniform [16,65536], Lambert, seed 3" % args.ndraws}
    if args.workload == "single":
        sc = scenes.single_large()
        nvis, area = scenes.visible_triangles(sc)
        return sc, {"workload": "single large draw: 1M indexed tris, 1920x1080, Lambert, back-face cull, seed 2",
                    "visible_triangles": nvis, "visible_mean_area_px": round(area, 3),
                    "calibration": "camera distance %.3f: the front-facing triangles inside the frustum average "
                                   "%.2f px" % (scenes.SINGLE_DISTANCE, area)}
    if args.workload == "soup":
        return scenes.small_soup(), {"workload": "plain single draw: 2048 tris, 256x256, seed 1"}
    if args.workload == "textured":
        return textured_scene(), {"workload": TEXTURED}
    return scenes.ordered_blend(), {"workload": "ordered blend: 200K tris, 1920x1080, SRC_ALPHA blend, seed 4"}


TEXTURED = ("textured: 200K tris (vertex radius log-uniform 0.004-0.08 NDC), 1920x1080, 1024x1024 RGBA8 combined "
            "image sampler, LINEAR / REPEAT, perspective-correct uv, seed 6")


def textured_scene():
    from kazan_gb300 import scenes
    return scenes.textured(seed=6, n=200_000, width=1920, height=1080, tex_w=1024, tex_h=1024, size_lo=0.004,
                           size_hi=0.08, linear=True)


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs"""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        """start sampling every 20 ms; returns once the first sample has arrived (or after 5 s)"""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return
        t0 = time.monotonic()
        while not self.lines and time.monotonic() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def window(self, t0, t1):
        """keep only the samples taken between t0 and t1 (monotonic seconds), plus the first one after t1
        so that a short timed region still has a sample that covers its end"""
        inside = [x for x in self.lines if t0 <= x[0] <= t1]
        after = [x for x in self.lines if x[0] > t1][:1]
        self.lines = inside + after

    def stop(self, t0=None, t1=None):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        if t0 is not None:
            self.window(t0, t1)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def profiled_traffic(workload, kernel):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu summary (None if absent)"""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(workload, {}).get(kernel)
    except (OSError, ValueError, AttributeError):
        return None


def profiled_instructions(workload, kernel):
    """warp instructions per launch of `kernel` on `workload` from the committed ncu summary (None if absent)"""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get("instructions", {}).get(workload, {}).get(kernel)
    except (OSError, ValueError, AttributeError):
        return None


def issue_roofline(workload, kernel, kernel_ms, sm_mhz):
    """the dominant kernel against the SMs' instruction issue rate (one warp instruction per cycle per
    scheduler, 4 schedulers per SM, at the SM clock measured during the timed region): its warp instructions
    per launch (ncu, committed) over its live CUDA-event duration; None without a profile"""
    import torch
    inst = profiled_instructions(workload, kernel)
    if not inst or not sm_mhz:
        return None
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    achieved = inst / (kernel_ms / 1e3) / 1e9
    peak = sms * 4 * sm_mhz * 1e6 / 1e9
    return {"achieved": round(achieved, 1), "peak": round(peak, 1), "unit": "G warp instructions/s",
            "frac": round(achieved / peak, 4), "warp_instructions": inst,
            "peak_source": "%d SMs x 4 schedulers x %.0f MHz (median SM clock under load)" % (sms, sm_mhz)}


def kernel_bytes(scene, kernel):
    """algorithmic HBM bytes of one launch of `kernel` over the whole scene (one segment):
      kz_k_persistent            the whole path: 12 T_indexed + S_v V + 64 draws + framebuffer traffic
      kz_k_vis_geometry / geometry  index + vertex-position bytes + push constants: 12 T_indexed + P V + 64 draws
                                 (P = 12 B position of the Lambert layout, 16 B of the colour layout)
      kz_k_vis_resolve           colour + depth stores: W H (4 + 4)
      kz_k_raster(_direct/_ds/_ms)  framebuffer read + write (depth written or not)
    returns (bytes, formula)"""
    t_idx = scene.triangles if scene.indexed else 0
    v = len(scene.vertices) if scene.indexed else 3 * scene.triangles
    push = 64 * len(scene.draws) if scene.shader == "lambert" else 0
    pos = 12 if scene.shader == "lambert" else 16
    wh = scene.width * scene.height
    if kernel in ("kz_k_vis_geometry", "kz_k_geometry"):
        return 12 * t_idx + pos * v + push, "12*T_indexed + %d*V + 64*draws" % pos
    if kernel == "kz_k_vis_resolve":
        return wh * 8, "W*H*(4+4)"
    if kernel in ("kz_k_raster", "kz_k_raster_direct", "kz_k_raster_ds", "kz_k_raster_ms"):
        return wh * ((4 + 4) * 2 if scene.depth_write else (2 * 4 + 4)), "W*H*framebuffer read+write"
    return scene.algorithmic_bytes(), "12*T_indexed + S_v*V + 64*draws + W*H*(4+4)*2"


def cpu_baseline(scene, budget_s=4.0):
    """the CPU oracle on a bounded prefix of the draws with all host threads; returns Mtris/s and sample"""
    from oracle import kz_oracle
    threads = os.cpu_count() or 1
    n = 1
    tri, el = 0, 0.0
    while True:
        draws = scene.draws[:n]
        t0 = time.perf_counter()
        kz_oracle.render(scene, threads=threads, draws=draws)
        el = time.perf_counter() - t0
        tri = sum(d.count for d in draws)
        if el > budget_s / 4 or n >= len(scene.draws):
            break
        n = min(len(scene.draws), max(n + 1, int(n * budget_s / 4 / max(el, 1e-3))))
    return {"value": tri / el / 1e6, "unit": "Mtris/s", "cores": threads, "kind": "port",
            "sample": "%d of %d draws (%d triangles), %.2f s wall; project CPU restatement (the reference "
                      "has no CPU rasteriser)" % (n, len(scene.draws), tri, el)}


def main():
    args = parse()
    from kazan_gb300 import replicas
    rk = replicas.from_env()
    rank, world, local = rk.rank, rk.world, rk.local
    if args.impl == "reference":
        if not rk.leader:
            return 0
        scene, cfg = make_scene(args)
        return reference_arm(args, scene, cfg)
    import torch
    torch.cuda.set_device(local)
    replicas.init(rk, "nccl", torch.device("cuda", local))
    if args.workload == "serve":
        return serve_main(args, rk)
    from kazan_gb300 import render
    scene, cfg = make_scene(args)
    indirect = None if args.indirect == "none" else args.indirect
    if indirect:
        cfg["workload"] = cfg["workload"].replace("vkCmdDrawIndexed", "vkCmdDrawIndexedIndirect") + \
            ", indirect commands in %s memory" % indirect
    r = render.Renderer()
    run = render.SceneRun(r, scene, host_visible=False, mode=args.mode, tile=args.tile, indirect=indirect)
    mode, tile, tuning = args.mode, args.tile, None
    if not args.no_tune:
        # launch schedule and tile side from the autotuner (measured here unless cached for this workload)
        from kazan_gb300 import autotune
        gpu = r.props.deviceName.decode(errors="replace")
        # blending, a D16 / D24S8 attachment or multisampling puts the pass on the ordered (tile) path
        ordered = scene.blend or scene.depth_format != "d32" or scene.samples > 1
        sig = autotune.signature(gpu, ordered, len(scene.draws), scene.triangles, scene.width, scene.height)
        sig += "|indirect" if indirect else ""
        sig += "" if (scene.depth_format, scene.samples) == ("d32", 1) else "|%s|%dx" % (scene.depth_format,
                                                                                        scene.samples)
        best, table = autotune.Tuner().choose(sig, autotune.scene_timer(run), autotune.candidates(ordered=ordered))
        mode, tile = best.mode, best.tile
        tuning = {"signature": sig, "chosen": best.options(),
                  "ms": None if table is None else {c.label(): round(v, 4) for c, v in table.items()}}
        # the chosen knobs hold for the command buffers recorded below
        for k in ("warp_px", "job_blocks", "geo_blocks"):
            r.drv.set_option(k, getattr(best, k))
    # two command buffers of the same draws: `graph_cb` is what an application submits (captured as a CUDA
    # graph at vkEndCommandBuffer, its kernels chained by programmatic dependent launch); `timed_cb`
    # launches its kernels at submit with an event pair around each launch, for the per-kernel times
    r.drv.set_option("mode", mode)
    r.drv.set_option("tile", tile)
    old_cb = run.cb
    graph_cb = run.record()
    r.drv.set_option("kernel_timing", 1)
    timed_cb = run.record()
    r.drv.set_option("kernel_timing", 0)
    r.free_command_buffer(old_cb)
    stream = torch.cuda.ExternalStream(r.stream())

    def barrier():
        replicas.barrier(rk)

    def timed_region(cb, run=run, steps=None):
        """K submissions of `cb` between a barrier + synchronize on both sides, timed by CUDA events on the
        queue stream; returns (ms per step over all ranks, clock record)"""
        steps = args.steps if steps is None else steps
        run.cb = cb
        for _ in range(max(3, args.warmup)):
            run.submit()
        r.drv.kernel_times(cb, reset=True)
        barrier()
        torch.cuda.synchronize()
        clocks = Clocks(local)
        clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.monotonic()
        e0.record(stream)
        for _ in range(steps):
            run.submit(wait=False)
        e1.record(stream)
        e1.synchronize()
        w1 = time.monotonic()
        r.drv.vkQueueWaitIdle(r.queue)
        ck = clocks.stop(w0, w1)
        torch.cuda.synchronize()
        barrier()
        return replicas.max_over_ranks(rk, e0.elapsed_time(e1) / steps, device="cuda"), ck

    # the headline: the application's command buffer
    ms, ck = timed_region(graph_cb)
    launches = run.stats().launches * args.steps
    # the same K submissions again with an event pair around each launch: per-kernel device time
    ms_k, ck_k = timed_region(timed_cb)
    ktimes = r.drv.kernel_times(timed_cb)
    run.cb = graph_cb
    r.free_command_buffer(timed_cb)
    kernels = {k: {"launches": n, "ms_per_launch": round(t / max(n, 1), 4),
                   "share": round(t / max(sum(x[0] for x in ktimes.values()), 1e-9), 4)}
               for k, (t, n) in ktimes.items()}
    dom = max(ktimes, key=lambda k: ktimes[k][0])
    dom_ms = ktimes[dom][0] / ktimes[dom][1]
    st = run.stats()
    tris = scene.triangles
    value = replicas.aggregate_rate(rk, tris, ms) / 1e6
    peak, peak_kind = measured_peak()
    kb, kformula = kernel_bytes(scene, dom)
    # the committed ncu figures hold for the default workloads only (the batched one at 4,096 draws)
    prof_key = args.workload if args.workload != "batched" or args.ndraws == 4096 else None
    achieved = kb / (dom_ms / 1e3) / 1e9
    out = {"metric": "Mtris/s (batched command buffer, exact coverage)", "value": round(value, 2),
           "unit": "Mtris/s", "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
           "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32+int64 (16.8 fixed-point edges)", "data": "synthetic (seeded scene generator)",
           "config": dict(cfg, tile=st.tile, mode=mode, triangles=tris,
                          l2="inputs larger than L2 (%.0f MB vertex+index per step)" % (
                              (scene.vertices.nbytes + (scene.indices.nbytes if scene.indices is not None else 0))
                              / 1e6), parallelism="replicas" if world > 1 else "single GPU"),
           "gfrag_per_s": round(st.fragments / (ms / 1e3) / 1e9, 3),
           "fragments": int(st.fragments),
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "traffic": profiled_traffic(prof_key, dom),
                        "kernel": dom, "kernel_ms": round(dom_ms, 4), "algorithmic_bytes": kb,
                        "bytes_formula": kformula,
                        "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                        "issue": issue_roofline(prof_key, dom, dom_ms, (ck_k or {}).get("sm_mhz"))},
           "kernels": kernels,
           "kernel_pass": {"ms_per_step": round(ms_k, 4), "steps": args.steps, "clocks": ck_k,
                           "how": "the same submissions with an event pair around each kernel launch"},
           "clocks": ck, "gpu_launches": int(launches), "autotune": tuning}
    if not args.no_perdraw:
        pd = render.SceneRun(r, scene, host_visible=False, mode="perdraw", tile=args.tile, indirect=indirect)
        pd.submit()
        steps = 2
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        p0.record(stream)
        for _ in range(steps):
            pd.submit(wait=False)
        p1.record(stream)
        p1.synchronize()
        r.drv.vkQueueWaitIdle(r.queue)
        pms = p0.elapsed_time(p1) / steps
        pst = pd.stats()
        out["per_draw"] = {"value": round(tris / (pms / 1e3) / 1e6, 2), "unit": "Mtris/s", "ms_per_step": round(pms, 3),
                           "launches_per_step": int(pst.launches), "steps": steps}
        out["batched_vs_per_draw"] = round(out["value"] / world / out["per_draw"]["value"], 2)
    # the graph-captured persistent form (one cooperative launch per submission), timed as the headline
    if mode == "persistent":
        pers_ms = ms
    else:
        r.drv.set_option("mode", "persistent")
        pcb = run.record()
        r.drv.set_option("mode", mode)
        pers_ms, _ = timed_region(pcb)
        run.cb = graph_cb
        r.free_command_buffer(pcb)
    out["persistent"] = {"value": round(replicas.aggregate_rate(rk, tris, pers_ms) / 1e6, 2), "unit": "Mtris/s",
                         "ms_per_step": round(pers_ms, 4), "steps": args.steps,
                         "how": "the same draws recorded in the persistent schedule, graph-launched"}
    if "per_draw" in out:
        out["persistent_vs_per_draw"] = round(out["persistent"]["value"] / world / out["per_draw"]["value"], 2)
    if not args.no_others and args.workload == "batched" and args.ndraws == 4096 and not indirect:
        out["other_workloads"] = other_workloads(r, render, timed_region, rk)
    if not args.no_e2e:
        import ctypes
        import numpy as np
        from kazan_gb300 import vk
        # two input/output sets used in turn, as a streaming application double-buffers: every step uploads
        # its vertex and index buffers from pinned host memory (the driver's host-visible memory), renders,
        # downloads its colour image and reads it on the host; the driver uploads on a copy engine, so one
        # step's upload overlaps the previous step's kernels.  Depth is scratch of the step (device-local).
        sets = [render.SceneRun(r, scene, host_visible=True, mode=mode, tile=tile, keep_mapped=True,
                                depth_host_visible=False, indirect=indirect) for _ in range(2)]
        fences = []
        for _ in range(2):
            f = ctypes.c_void_p()
            fci = vk.VkFenceCreateInfo(vk.ST_FENCE_CREATE_INFO, None, 0)
            vk.check("vkCreateFence", r.drv.vkCreateFence(r.device, ctypes.byref(fci), None, ctypes.byref(f)))
            fences.append(f)
        ptrs = [r.map(e.color) for e in sets]
        nbytes = sets[0].color.pitch * scene.height
        host = np.empty(nbytes, dtype=np.uint8)

        def finish(k):
            arr = (ctypes.c_void_p * 1)(fences[k % 2])
            vk.check("vkWaitForFences", r.drv.vkWaitForFences(r.device, 1, arr, 1, 60_000_000_000))
            vk.check("vkResetFences", r.drv.vkResetFences(r.device, 1, arr))
            ctypes.memmove(host.ctypes.data, ptrs[k % 2], nbytes)

        for e in sets:
            e.submit()
        steps = max(4, min(args.steps, 10))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(steps):
            r.submit(sets[k % 2].cb, fences[k % 2])
            if k >= 1:
                finish(k - 1)
        finish(steps - 1)
        el = replicas.max_over_ranks(rk, (time.perf_counter() - t0) / steps, device="cuda")
        for f in fences:
            r.drv.vkDestroyFence(r.device, f, None)
        h2d = scene.vertices.nbytes + (scene.indices.nbytes if scene.indices is not None else 0)
        out["e2e"] = {"value": round(tris * world / el / 1e6, 2), "unit": "Mtris/s", "h2d_bytes_per_step": int(h2d),
                      "d2h_bytes_per_step": int(nbytes), "ms_per_step": round(el * 1e3, 3), "steps": steps,
                      "pipelining": "two input/output sets in turn; uploads on the driver's copy stream"}
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(scene)
    if rank == 0:
        print(json.dumps(out), flush=True)
    r.close()
    replicas.finish(rk)
    return 0


def other_workloads(r, render, timed_region, rk):
    """short timings of the other render configurations (seeded synthetic scenes): each recorded in the
    batched schedule at tile 16 with the visibility path's default knobs and graph-launched for a few hundred
    milliseconds, then once more with kernel timing on for the dominant kernel; device-resident inputs"""
    from kazan_gb300 import autotune, scenes
    out = {}
    for k, v in autotune.DEFAULTS.items():
        r.drv.set_option(k, v)
    cases = [("plain small draw: 2,048 non-indexed tris, 256x256, seed 1", scenes.small_soup(), 2000),
             ("single large draw: 1M indexed tris, 1920x1080, Lambert, back-face cull, seed 2", scenes.single_large(),
              800),
             ("ordered blend: 200K tris, 1920x1080, SRC_ALPHA / ONE_MINUS_SRC_ALPHA, depth writes off, seed 4",
              scenes.ordered_blend(), 100),
             (TEXTURED, textured_scene(), 400)]
    for name, scene, steps in cases:
        r.drv.set_option("mode", "batched")
        r.drv.set_option("tile", 16)
        run = render.SceneRun(r, scene, host_visible=False, mode="batched", tile=16)
        ms, ck = timed_region(run.cb, run=run, steps=steps)
        st = run.stats()
        r.drv.set_option("kernel_timing", 1)
        tcb = run.record()
        r.drv.set_option("kernel_timing", 0)
        timed_region(tcb, run=run, steps=steps)
        kt = r.drv.kernel_times(tcb)
        total = sum(t for t, _ in kt.values())
        dom = max(kt, key=lambda k: kt[k][0])
        row = {"ms_per_step": round(ms, 4), "mtris_per_s": round(scene.triangles / (ms / 1e3) / 1e6, 2),
               "gfrag_per_s": round(st.fragments / (ms / 1e3) / 1e9, 3), "fragments": int(st.fragments),
               "triangles": scene.triangles, "dominant_kernel": dom, "dominant_share": round(kt[dom][0] / total, 4),
               "clocks": ck}
        if scene.shader == "lambert":
            nvis, area = scenes.visible_triangles(scene)
            row["visible_triangles"] = nvis
            row["visible_mean_area_px"] = round(area, 3)
        out[name] = row
        r.free_command_buffer(tcb)
    out.update(serving_summary(r))
    return out


def serving_summary(r, rate=5000, n=1500):
    """the serving configuration at one rate of the configured sweep: 64 clients with resident scenes, the
    same Poisson request stream served batched and one request at a time (latency arrival -> fence)"""
    from kazan_gb300 import serving
    t0 = time.perf_counter()
    backend = serving.VulkanBackend(r, serving.client_specs(), mode="batched")
    setup_s = time.perf_counter() - t0
    admitted, resident = serving.admit(backend.sizes, 40e9)
    for i in admitted:  # warm-up: every command buffer once
        backend.wait(backend.submit([serving.Request(i, 0, 0.0, res, serving.TMAX)
                                     for res in range(len(serving.RESOLUTIONS))]))
    b, one = serving.sweep(backend, admitted, [rate], n)
    backend.close()
    name = ("serving: 64 clients, Poisson arrivals at %d req/s, %d requests, each with its own resolution "
            "(256^2..1920x1080), triangle count (log-uniform 1K-500K) and camera" % (rate, n))
    return {name: {"admitted_clients": len(admitted), "resident_gb": round(resident / 1e9, 3),
                   "setup_s": round(setup_s, 2), "batched": b[0].as_dict(), "one_at_a_time": one[0].as_dict()}}


def serve_main(args, rk):
    """the serving configuration: 64 clients with resident scenes, Poisson arrivals swept over rates;
    batched submissions against one request at a time on the same request streams"""
    from kazan_gb300 import render, replicas, serving
    r = render.Renderer()
    specs = serving.client_specs()
    t0 = time.perf_counter()
    backend = serving.VulkanBackend(r, specs, mode=args.mode)
    setup_s = time.perf_counter() - t0
    admitted, resident = serving.admit(backend.sizes, args.budget_gb * 1e9)
    for i in admitted:  # warm-up: every command buffer once
        backend.wait(backend.submit([serving.Request(i, 0, 0.0, res, serving.TMAX)
                                     for res in range(len(serving.RESOLUTIONS))]))
    rates = [100, 250, 500, 1000, 2500, 5000, 10000, 20000, 40000]  # the configured sweep, then past saturation
    clocks = Clocks(rk.local)
    clocks.start()
    w0 = time.monotonic()
    rows, best = [], None
    for rate in rates:
        n = int(min(3000, max(200, rate * 1.5)))
        b, one = serving.sweep(backend, admitted, [rate], n)
        b, one = b[0], one[0]
        rows.append({"rate_req_per_s": rate, "requests": n, "batched": b.as_dict(), "one_at_a_time": one.as_dict()})
        print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
        best = b
    ck = clocks.stop(w0, time.monotonic())
    launches = sum(r.drv.stats(backend.runs[i][0].cb).launches for i in admitted) / max(1, len(admitted))
    value = replicas.aggregate_rate(rk, best.mtris_per_s * best.wall_s * 1e6, replicas.max_over_ranks(
        rk, best.wall_s * 1e3, device="cuda")) / 1e6
    out = {"metric": "Mtris/s (serving: 64 clients, Poisson arrivals, batched submissions)", "value": round(value, 2),
           "unit": "Mtris/s", "n_gpus": rk.world, "steps": len(rates), "warmup": 1,
           "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32+int64 (16.8 fixed-point edges)", "data": "synthetic (seeded scene generator)",
           "config": {"workload": "serving: 64 clients, Poisson arrivals; per request a resolution uniform over "
                                  "256^2/512^2/1024^2/1920x1080, a triangle count log-uniform in [1K, 500K] (a "
                                  "prefix of the client's resident 500K-triangle sphere mesh) and its own random MVP "
                                  "(uniform buffer + indirect command written per request)",
                      "mode": args.mode, "budget_gb": args.budget_gb, "admitted_clients": len(admitted),
                      "resident_gb": round(resident / 1e9, 3), "setup_s": round(setup_s, 2),
                      "max_batch": 64, "max_inflight": 4, "value_at_rate": rates[-1],
                      "configured_rates": [100, 250, 500, 1000, 2500, 5000],
                      "l2": "resident scenes of all clients (resident_gb) rendered in turn"},
           "serving": rows,
           "e2e": {"value": round(value, 2), "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                   "note": "latency is host-measured arrival -> fence; scenes are resident by design"},
           "roofline": None, "clocks": ck, "gpu_launches": int(launches * best.served)}
    if rk.leader:
        print(json.dumps(out), flush=True)
    backend.close()
    r.close()
    replicas.finish(rk)
    return 0


def reference_arm(args, scene, cfg):
    """the reference arm: the CPU implementation of this path (the project's oracle port, since the reference
    driver's draw path is unimplemented) on the host cores, each step a bounded sample of the workload"""
    from oracle import kz_oracle
    threads = os.cpu_count() or 1
    cb = cpu_baseline(scene)
    n = int(cb["sample"].split(" of ")[0])
    draws = scene.draws[:n]
    tri = sum(d.count for d in draws)
    for _ in range(args.warmup):
        kz_oracle.render(scene, threads=threads, draws=draws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        kz_oracle.render(scene, threads=threads, draws=draws)
    el = (time.perf_counter() - t0) / args.steps
    v = tri / el / 1e6
    out = {"impl": "reference", "metric": "Mtris/s (batched command buffer, exact coverage)", "value": round(v, 3),
           "unit": "Mtris/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(el * 1e3, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32+int64 (16.8 fixed-point edges)", "data": "synthetic (seeded scene generator)",
           "config": dict(cfg, sample_draws=n, sample_triangles=tri),
           "cpu_baseline": {"value": round(v, 3), "unit": "Mtris/s", "cores": threads, "kind": "port",
                            "sample": "%d of %d draws (%d triangles) per step; project CPU restatement, the reference "
                                      "has no CPU rasteriser (vulkan-driver/src/api_impl.rs:4632-4653)"
                                      % (n, len(scene.draws), tri)},
           "e2e": {"value": round(v, 3), "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
