"""Benchmark: forward+backward of the render path, 1M Gaussians at 1920x1080.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--scene hd|uhd|small|batch|fit|warmstart|netstep] [--no-cpu-baseline]

One step = project -> sort/bin -> rasterize forward with the L2 loss against
a target image -> rasterize backward -> project backward (one CUDA graph, the
intersection count kept on the device), on seeded synthetic inputs with the
benchmark scene's shapes and distributions.

* ``value``: ms per step with inputs resident in HBM, CUDA events on the
  launching stream, L2 flushed (a 256 MiB write) before every timed step and
  excluded from the timing.
* ``e2e``: the same step with the inputs copied from pinned host memory and
  the loss and the five gradient arrays copied back inside the timed region,
  one step at a time (``RenderSession.step_io``), with the host link's
  measured bandwidth (``link_gbs``).
* ``e2e_streamed``: consecutive steps through ``stream_step`` (every step
  still uploads its inputs and downloads its results; double-buffered, so
  the copies of neighbouring steps overlap the computation).
* ``roofline``: the dominant kernel against its binding floor -- for the
  rasterizers FP32 FLOPs (or ex2 results) over its time against the nominal
  rate at the sampled clock, with the HBM fraction (algorithmic bytes over
  the measured copy bandwidth) and its ncu DRAM traffic beside it; ``pairs``
  and ``stage_roofline``: work counts and each stage's HBM / FP32 / ex2 floor.
* ``--impl reference``: the reference's own CUDA kernels (built from its
  sources into oracle/_ref) driven with its stock host orchestration
  (oracle/ref_harness.cu) on the same GPU, same workload; when those are not
  built, the CPU restatement in oracle/ (all host threads) stands in.

Multi-GPU (torchrun): every rank runs an independent replica of the
workload (the render path has no exchange step); the timing is max over
ranks and ``value`` is the whole-job time per step (elapsed / (K * N)).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+bwd ms/iter, 1M Gaussians @1080p"
UNIT = "ms"
L2_FLUSH_BYTES = 256 << 20

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the dominant kernel on the 1M-Gaussian 1920x1080 scene, from one ncu
# capture of that launch (104.46 MB read + 4.77 MB written).
NCU_TRAFFIC = {"raster_bwd": 104_461_312 + 4_772_352}
# The batched backward captured at a quarter of the batch's Gaussian counts:
# bytes read, bytes written, intersections.
NCU_BATCH_QUARTER = {"raster_bwd": (1_292_425_472, 109_377_536, 23_673_320)}


def radix_passes(bits: int) -> int:
    """Onesweep passes over `bits` key bits (8 per pass)."""
    return (max(1, bits) + 7) // 8


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)
            self.t.join(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
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
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# workloads

class OursStep:
    """The render path through libsplat's C ABI, as one preallocated,
    sync-free step (jaxsplat_gb300.RenderSession) replayed as a CUDA graph."""

    # the L2 loss runs inside the forward rasterizer; the packing pass runs on
    # a second stream during the sort
    STAGES = ["project_fwd", "sort", "raster_fwd", "raster_bwd", "project_bwd", "end"]

    def __init__(self, sc, dev, graph=True):
        import torch

        from jaxsplat_gb300.session import RenderSession

        self.torch, self.sc, self.dev = torch, sc, dev
        kw = sc.kwargs
        self.sess = RenderSession(sc.spec.num_points, img_shape=kw["img_shape"], f=kw["f"],
                                  c=kw["c"], glob_scale=kw["glob_scale"],
                                  clip_thresh=kw["clip_thresh"], block_size=sc.spec.block_width,
                                  device=dev)
        # inputs and outputs as single pinned blocks: one H2D and one D2H copy
        # per step
        self.host_in = self.sess.host_inputs(
            *(getattr(sc, k) for k in ("means3d", "scales", "quats", "colors", "opacities",
                                       "viewmat", "background", "target")))
        self.host_out = torch.empty(self.sess.outputs.numel(), dtype=torch.float32,
                                    pin_memory=True)
        self.h2d_bytes = self.host_in.numel() * 4
        self.d2h_bytes = self.host_out.numel() * 4
        self.upload()
        self.count = self.sess.measure_capacity()
        self.graph = graph
        if graph:
            self.sess.capture()
            self.sess.capture_io(self.host_in, self.host_out)
        h, w = kw["img_shape"]
        bw = sc.spec.block_width
        tiles = ((w + bw - 1) // bw) * ((h + bw - 1) // bw)
        tile_passes = radix_passes(max(1, (tiles - 1).bit_length()))
        # project (+ packing), depth keys (+ digit counts), 4-pass depth sort,
        # emission (offsets, expansion + digit counts), tile sort, bins,
        # raster fwd (+ loss), raster bwd, project bwd
        self.kernels_per_step = 1 + 1 + 4 + 2 + tile_passes + 1 + 1 + 1 + 1
        self.passes = tile_passes

    def launches_per_step(self):
        return self.kernels_per_step

    def stage_bytes(self):
        """Algorithmic bytes per stage.  Raster backward: 52 B per
        intersection, 32 B per pixel and 9 fp32 atomics (36 B) per
        contributing (tile, Gaussian) pair I_c, counted by splat_count_pairs
        (`pairs`, when taken); raster forward: 40 B per intersection and 20 B
        per pixel, plus the fused L2 loss (target in, v_img out: 24 B per
        pixel); the projection also writes the packed records (16 B more in,
        48 B more out per Gaussian)."""
        n, I = self.sc.spec.num_points, self.count
        h, w = self.sc.spec.img_shape
        P = h * w
        ic = (getattr(self, "pairs", None) or {}).get("tile_gaussian_contributing", 0)
        return {"raster_bwd": 52 * I + 32 * P + 36 * ic, "raster_fwd": 40 * I + 44 * P,
                "sort": 16 * n * 4 + 28 * n + 8 * I + 16 * I * self.passes,
                "project_fwd": 164 * n, "project_bwd": 140 * n}

    def ncu_traffic(self, kernel):
        """Measured DRAM bytes of one launch (ncu), for the 1080p scene only."""
        if self.sc.spec.name != "hd" or kernel not in NCU_TRAFFIC:
            return None, None
        return NCU_TRAFFIC[kernel], "ncu capture of this workload"

    def step(self, ev=None):
        if ev is not None:
            self.sess.step(mark=lambda name: ev[name].record())
        elif self.graph:
            self.sess.replay()
        else:
            self.sess.step()
        g = self.sess.grads
        return self.sess.loss, [g["means3d"], g["scales"], g["quats"], g["colors"],
                                g["opacities"]]

    def upload(self):
        self.sess.upload(self.host_in)

    def download(self):
        self.sess.download(self.host_out)

    def step_e2e(self):
        """Host input block to host output block with the copies overlapped
        (RenderSession.step_io, as a graph)."""
        if self.graph:
            self.sess.replay_io()
        else:
            self.sess.step_io(self.host_in, self.host_out)


class RefStep:
    """The reference's kernels through its four custom calls (oracle/ref.py)."""

    def __init__(self, sc, dev):
        import torch

        from oracle.ref import RefKernels

        self.torch, self.sc, self.dev = torch, sc, dev
        self.rk = RefKernels()
        self.kw = dict(sc.kwargs, block_width=sc.spec.block_width)
        self.host = {k: torch.from_numpy(getattr(sc, k)).pin_memory()
                     for k in ("means3d", "scales", "quats", "colors", "opacities", "viewmat",
                               "background", "target")}
        self.d = {k: v.to(dev) for k, v in self.host.items()}
        n = sc.spec.num_points
        self.zn = torch.zeros(n, 1, device=dev)
        h, w = self.kw["img_shape"]
        self.zalpha = torch.zeros(h, w, 1, device=dev)

    def launches_per_step(self):
        return 0

    def step(self, ev=None):
        rk, d, kw = self.rk, self.d, self.kw
        ikw = dict(img_shape=kw["img_shape"], block_width=kw["block_width"])
        p = rk.project_fwd(d["means3d"], d["scales"], d["quats"], d["viewmat"], **kw)
        r = rk.rasterize_fwd(d["colors"], d["opacities"], d["background"], p["xys"],
                             p["depths"], p["radii"], p["conics"], p["cum_tiles_hit"], **ikw)
        img = r["img"]
        loss = ((img - d["target"]) ** 2).mean()
        v_img = (2.0 * (img - d["target"]) / img.numel()).contiguous()
        rb = rk.rasterize_bwd(d["colors"], d["opacities"], d["background"], p["xys"],
                              p["depths"], p["radii"], p["conics"], p["cum_tiles_hit"],
                              r["final_Ts"], r["final_idx"], v_img, self.zalpha, **ikw)
        pb = rk.project_bwd(d["means3d"], d["scales"], d["quats"], d["viewmat"], p["cov3d"],
                            p["xys"], p["radii"], p["conics"], p["compensation"], self.zn,
                            rb["v_xy"], self.zn, rb["v_conic"], **kw)
        return loss, [pb["v_mean3d"], pb["v_scale"], pb["v_quat"], rb["v_colors"],
                      rb["v_opacity"]]

    def upload(self):
        for k, v in self.host.items():
            self.d[k].copy_(v, non_blocking=True)


class BatchStep:
    """The batched workload: 4 scenes x 8 views with mixed image sizes, all
    views in one pass of each kernel (jaxsplat_gb300.BatchSession), one CUDA
    graph per step."""

    STAGES = OursStep.STAGES

    def __init__(self, seed, dev, graph=True, autotune=False, log=None, points=None):
        import torch

        from jaxsplat_gb300.batch import BatchSession
        from jaxsplat_gb300.scenes import BATCH_POINTS, make_batch

        self.torch, self.dev = torch, dev
        scenes, views, targets = make_batch(seed, scene_points=points or BATCH_POINTS)
        self.views = views
        self.sess = BatchSession(scenes, views, targets, block_size=16, chunk=1, device=dev)
        self.tuning = None
        if autotune:
            self.tuning = self.sess.autotune(log=log)
        s = self.sess
        # the step's inputs and outputs as single pinned blocks (one copy each)
        self.host_in = s.inputs.cpu().pin_memory()
        self.host_out = torch.empty(s.outputs.numel(), dtype=torch.float32, pin_memory=True)
        self.h2d_bytes = self.host_in.numel() * 4
        self.d2h_bytes = self.host_out.numel() * 4
        self.count = s.measure_capacity()
        self.graph = graph
        if graph:
            s.capture()
            s.capture_io(self.host_in, self.host_out)
        b = s.batch
        tile_passes = radix_passes(max(1, (int(b.num_tiles) - 1).bit_length()))
        # project, depth keys (+ digit counts), 4-pass depth sort, emission
        # (2, + digit counts), tile sort, bins, tile costs, 3-pass cost sort
        # (+ hist), raster fwd (+ loss), raster bwd, project bwd; the
        # projection writes the packed records
        self.kernels_per_step = 1 + 1 + 4 + 2 + tile_passes + 1 + 1 + 4 + 1 + 1 + 1
        self.passes = tile_passes

    def launches_per_step(self):
        return self.kernels_per_step

    def stage_bytes(self):
        """As OursStep.stage_bytes over E (view, Gaussian) entries, without the
        atomics term (no pair count for batches: a lower bound)."""
        b, I = self.sess.batch, self.count
        E, P = int(b.num_entries), int(b.num_pixels)
        return {"raster_bwd": 52 * I + 32 * P, "raster_fwd": 40 * I + 44 * P,
                "sort": 16 * E * 4 + 28 * E + 8 * I + 16 * I * self.passes,
                "project_fwd": 164 * E, "project_bwd": 140 * E}

    def ncu_traffic(self, kernel):
        """DRAM bytes of one launch scaled from the quarter-size capture: the
        per-pixel reads (final_Ts, final_idx, v_img, v_img_alpha: 24 B per
        pixel, the same pixels at every scale) stay, the rest (records,
        lists, gradient writes) scales with the intersections."""
        if kernel not in NCU_BATCH_QUARTER:
            return None, None
        rd, wr, iq = NCU_BATCH_QUARTER[kernel]
        pix = 24 * int(self.sess.batch.num_pixels)
        est = pix + (rd + wr - pix) * self.count / iq
        return int(est), "quarter-size ncu capture, non-pixel bytes scaled by intersections"

    def step(self, ev=None):
        if ev is not None:
            self.sess.step(mark=lambda name: ev[name].record())
        elif self.graph:
            self.sess.replay()
        else:
            self.sess.step()
        s = self.sess
        return s.loss, [s.v_mean3d, s.v_scale, s.v_quat, s.v_colors, s.v_opacity]

    def upload(self):
        self.sess.upload(self.host_in)

    def download(self):
        self.sess.download(self.host_out)

    def step_e2e(self):
        """Host blocks in and out with the copies overlapped
        (BatchSession.step_io, as a graph)."""
        if self.graph:
            self.sess.replay_io()
        else:
            self.sess.step_io(self.host_in, self.host_out)


class RefBatchStep:
    """The batched workload through the reference's kernels the way a
    jaxsplat user runs it: one render call per view, scene gradients summed
    over the views."""

    def __init__(self, seed, dev, points=None):
        import torch

        from jaxsplat_gb300.scenes import BATCH_POINTS, make_batch
        from oracle.ref import RefKernels

        self.torch, self.dev = torch, dev
        self.rk = RefKernels()
        scenes, views, targets = make_batch(seed, scene_points=points or BATCH_POINTS)
        self.views = views
        self.host = {}
        for i, x in enumerate(scenes):
            for k, v in x.items():
                self.host[f"{i}:{k}"] = torch.from_numpy(np.ascontiguousarray(v)).pin_memory()
        for i, t in enumerate(targets):
            self.host[f"t{i}"] = torch.from_numpy(t).pin_memory()
        self.d = {k: v.to(dev) for k, v in self.host.items()}
        self.scenes = [{k: self.d[f"{i}:{k}"] for k in x} for i, x in enumerate(scenes)]
        self.targets = [self.d[f"t{i}"] for i in range(len(targets))]
        self.vm = [torch.from_numpy(v["viewmat"]).to(dev) for v in views]
        self.bg = [torch.from_numpy(np.asarray(v["background"], np.float32)).to(dev) for v in views]

    def launches_per_step(self):
        return 0

    def step(self, ev=None):
        torch, rk = self.torch, self.rk
        loss = 0.0
        grads = [[torch.zeros_like(x[k]) for k in ("means3d", "scales", "quats", "colors",
                                                     "opacities")] for x in self.scenes]
        for k, v in enumerate(self.views):
            d = self.scenes[v["scene"]]
            h, w = v["img_shape"]
            kw = dict(img_shape=(h, w), f=v["f"], c=v["c"], glob_scale=1.0, clip_thresh=0.01,
                      block_width=16)
            ikw = dict(img_shape=(h, w), block_width=16)
            zn = torch.zeros(d["means3d"].shape[0], 1, device=self.dev)
            p = rk.project_fwd(d["means3d"], d["scales"], d["quats"], self.vm[k], **kw)
            r = rk.rasterize_fwd(d["colors"], d["opacities"], self.bg[k], p["xys"], p["depths"],
                                 p["radii"], p["conics"], p["cum_tiles_hit"], **ikw)
            img = r["img"]
            loss = loss + ((img - self.targets[k]) ** 2).mean()
            v_img = (2.0 * (img - self.targets[k]) / img.numel()).contiguous()
            rb = rk.rasterize_bwd(d["colors"], d["opacities"], self.bg[k], p["xys"], p["depths"],
                                  p["radii"], p["conics"], p["cum_tiles_hit"], r["final_Ts"],
                                  r["final_idx"], v_img, torch.zeros(h, w, 1, device=self.dev),
                                  **ikw)
            pb = rk.project_bwd(d["means3d"], d["scales"], d["quats"], self.vm[k], p["cov3d"],
                                p["xys"], p["radii"], p["conics"], p["compensation"], zn,
                                rb["v_xy"], zn, rb["v_conic"], **kw)
            for acc, g in zip(grads[v["scene"]], (pb["v_mean3d"], pb["v_scale"], pb["v_quat"],
                                                   rb["v_colors"], rb["v_opacity"])):
                acc += g
        return loss, [g for sc in grads for g in sc]

    def upload(self):
        for k, v in self.host.items():
            self.d[k].copy_(v, non_blocking=True)


# ---------------------------------------------------------------------------

def time_device(st, steps, warmup, flush):
    """Per-step CUDA-event timing, L2 flushed before each step (untimed)."""
    torch = st.torch
    for _ in range(warmup):
        st.step()
    torch.cuda.synchronize()
    total = 0.0
    for _ in range(steps):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        st.step()
        b.record()
        torch.cuda.synchronize()
        total += a.elapsed_time(b)
    return total


def time_stages(st, steps, flush):
    """The same step run eagerly with an event before each stage (per-stage
    device time for the roofline)."""
    torch = st.torch
    names = st.STAGES
    stages = {}
    for _ in range(steps):
        flush.fill_(1)
        ev = {k: torch.cuda.Event(enable_timing=True) for k in names}
        st.step(ev)
        torch.cuda.synchronize()
        for x, y in zip(names, names[1:]):
            stages[x] = stages.get(x, 0.0) + ev[x].elapsed_time(ev[y])
    return {k: v / steps for k, v in stages.items()}


def link_bandwidth(dev, nbytes=256 << 20, reps=3):
    """Host link bandwidth of this machine, GB/s: one pinned 256 MB copy each
    way, best of `reps` (measured outside the timed regions; it bounds e2e)."""
    import torch

    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = round(nbytes / (best * 1e-3) / 1e9, 1)
    return out


def time_e2e(st, steps, flush):
    """Host buffers: H2D of the inputs and D2H of loss + gradients inside.
    Steps with `download()` move their outputs as one block; the others copy
    the loss and each gradient."""
    torch = st.torch
    out_host = None
    total = 0.0
    bi = getattr(st, "h2d_bytes", None)
    if bi is None:
        bi = sum(v.numel() * v.element_size() for v in st.host.values())
    bo = getattr(st, "d2h_bytes", 0)
    if hasattr(st, "step_e2e"):
        st.step_e2e()  # untimed warm-up of the copy graph
        torch.cuda.synchronize()
    for _ in range(steps):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        if hasattr(st, "step_e2e"):
            st.step_e2e()
            b.record()
            torch.cuda.synchronize()
            total += a.elapsed_time(b)
            continue
        st.upload()
        loss, grads = st.step()
        if hasattr(st, "download"):
            st.download()
        else:
            outs = [loss] + grads
            if out_host is None:
                out_host = [torch.empty(o.shape, dtype=o.dtype, pin_memory=True) for o in outs]
                bo = sum(o.numel() * o.element_size() for o in outs)
            for h, o in zip(out_host, outs):
                h.copy_(o.reshape(h.shape), non_blocking=True)
        b.record()
        torch.cuda.synchronize()
        total += a.elapsed_time(b)
    return total / steps, bi, bo


def time_e2e_streamed(st, steps, flush):
    """Consecutive steps through RenderSession.stream_step: each step's inputs
    go host -> device and its loss and gradients device -> host, double
    buffered so that step i+1's upload and step i's download overlap step i's
    computation.  The L2 flush before every step runs on the compute stream,
    inside the timed region, and so do the first step's upload and the last
    step's download, which nothing overlaps (fill and drain of the pipeline,
    amortised over the steps)."""
    torch = st.torch
    sess = st.sess
    sess.capture_stream()
    for _ in range(3):  # warm-up
        flush.fill_(1)
        sess.stream_step(st.host_in, st.host_out)
    sess.stream_sync()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        flush.fill_(1)
        sess.stream_step(st.host_in, st.host_out)
    sess.stream_sync()
    b.record()
    torch.cuda.synchronize()
    sess.check()
    return {"value": round(a.elapsed_time(b) / steps, 4), "unit": UNIT,
            "h2d_bytes_per_step": st.h2d_bytes, "d2h_bytes_per_step": st.d2h_bytes,
            "steps": steps,
            "mode": "stream_step: every step uploads its inputs and downloads its "
                    "loss and gradients; double-buffered, so step i+1's upload and step i's "
                    "download run while step i computes; L2 flush inside the timed region"}


def cpu_baseline(sc):
    """The CPU restatement (oracle/, fp32, all host threads) on one step of
    the same workload."""
    from oracle.oracle import Oracle

    o = Oracle("f32")
    threads = len(os.sched_getaffinity(0))
    o.set_threads(threads)
    kw = sc.kwargs
    bw = sc.spec.block_width
    args = (sc.means3d, sc.scales, sc.quats, sc.colors, sc.opacities)
    fwd = o.render(*args, viewmat=sc.viewmat, background=sc.background, block_size=bw, **kw)
    v_img = (2.0 * (fwd["img"] - sc.target) / fwd["img"].size).astype(np.float32)
    t = time.perf_counter()
    o.render(*args, viewmat=sc.viewmat, background=sc.background, block_size=bw, v_img=v_img,
             **kw)
    dt = time.perf_counter() - t
    return {"value": round(dt * 1000.0, 1), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"one forward+backward step of the full {sc.spec.name} scene "
                      f"({sc.spec.num_points} Gaussians, {kw['img_shape'][1]}x{kw['img_shape'][0]};"
                      " fp32 CPU restatement, OpenMP over tiles and Gaussians)"}


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The slowest replica's time (the whole job waits for it)."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_ms_per_step(total_ms: float, steps: int, world: int) -> float:
    """Replicas each run `steps` steps in `total_ms` (max over ranks), so the
    job completes world * steps steps in that time."""
    return total_ms / (steps * world)


def add_stages_and_roofline(line, st, steps, flush):
    stage_ms = time_stages(st, max(3, steps // 5), flush)
    line["stages_ms"] = {k: round(v, 4) for k, v in stage_ms.items()}
    line["num_intersects"] = st.count
    stage_ms.pop("end", None)
    dominant = max(stage_ms, key=stage_ms.get)
    bytes_by_stage = st.stage_bytes()
    peak, src = _peaks()
    achieved = bytes_by_stage[dominant] / (stage_ms[dominant] * 1e-3) / 1e9
    traffic, traffic_src = st.ncu_traffic(dominant)
    line["roofline"] = {"kernel": dominant, "bound": "hbm", "achieved": round(achieved, 1),
                        "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                        "peak_source": src, "traffic": traffic,
                        "algorithmic_bytes": bytes_by_stage[dominant]}
    if traffic is not None:
        line["roofline"]["traffic_source"] = traffic_src


# Nominal per-SM rates of sm_103a: 128 FP32 lanes (an FMA counts as 2
# FLOPs) and 16 MUFU ex2 results per clock.  Scaled by the SM count and the SM
# clock sampled during the run.
FP32_FLOPS_PER_SM_CLK = 256
EX2_PER_SM_CLK = 16
# FP32 operations per evaluated pixel-Gaussian pair (falloff, exponent,
# alpha, blend) and the further ones per contributing pair in the backward
# (transmittance, colour, alpha, conic and position cotangents).
FLOPS_PER_EVAL = 15
FLOPS_PER_CONTRIB_BWD = 30


def add_compute_roofline(line, st):
    """Per-stage floors from the step's own work counts: HBM bytes over the
    measured copy bandwidth for every stage; for the rasterizers also FP32
    FLOPs and ex2 counts over the nominal rates (from splat_count_pairs).
    `step.frac` = the sum of the stage floors over the measured step time."""
    import torch

    pairs = st.pairs
    line["pairs"] = pairs
    peak, src = _peaks()
    props = torch.cuda.get_device_properties(st.dev)
    clk = (line.get("clocks") or {}).get("sm_mhz") or (line.get("clocks") or {}).get("sm_max_mhz")
    if not clk:
        return
    sms = props.multi_processor_count
    fp32 = sms * FP32_FLOPS_PER_SM_CLK * clk * 1e6
    ex2 = sms * EX2_PER_SM_CLK * clk * 1e6
    work = st.stage_bytes()
    flops = {"raster_fwd": FLOPS_PER_EVAL * pairs["fwd_evaluated"],
             "raster_bwd": FLOPS_PER_EVAL * pairs["bwd_evaluated"]
             + FLOPS_PER_CONTRIB_BWD * pairs["bwd_contributing"]}
    sfu = {"raster_fwd": pairs["fwd_evaluated"], "raster_bwd": pairs["bwd_evaluated"]}
    stages, total_floor = {}, 0.0
    for name, ms in line["stages_ms"].items():
        if name not in work:
            continue
        floors = {"hbm": work[name] / (peak * 1e9) * 1e3}
        if name in flops:
            floors["fp32"] = flops[name] / fp32 * 1e3
            floors["sfu"] = sfu[name] / ex2 * 1e3
        bound = max(floors, key=floors.get)
        total_floor += floors[bound]
        stages[name] = {"ms": ms, "floor_ms": round(floors[bound], 4), "bound": bound,
                        "frac": round(floors[bound] / ms, 4)}
    # the headline roofline of the dominant kernel names its binding floor:
    # for the rasterizers that is FP32 (or ex2) issue, not HBM; the HBM
    # fraction stays beside it
    dom = line.get("roofline", {}).get("kernel")
    if dom in stages and stages[dom]["bound"] != "hbm":
        b = stages[dom]["bound"]
        ms = line["stages_ms"][dom]
        hbm = {k: line["roofline"][k] for k in ("achieved", "peak", "unit", "frac", "peak_source")}
        if b == "fp32":
            achieved, cpeak, unit = flops[dom] / (ms * 1e-3) / 1e12, fp32 / 1e12, "TFLOP/s"
        else:
            achieved, cpeak, unit = sfu[dom] / (ms * 1e-3) / 1e12, ex2 / 1e12, "Tex2/s"
        line["roofline"].update({
            "bound": b, "achieved": round(achieved, 3), "peak": round(cpeak, 2), "unit": unit,
            "frac": round(achieved / cpeak, 4),
            "peak_source": f"nominal per-SM rate x {sms} SMs x {clk:.0f} MHz (sampled)",
            "algorithmic_flops" if b == "fp32" else "algorithmic_ex2":
                flops[dom] if b == "fp32" else sfu[dom],
            "hbm": hbm})
    line["stage_roofline"] = {
        "stages": stages,
        "step": {"floor_ms": round(total_floor, 4), "ms": line["value"],
                 "frac": round(total_floor / line["value"], 4)},
        "peaks": {"hbm_gbs": peak, "hbm_source": src,
                  "fp32_tflops": round(fp32 / 1e12, 1), "ex2_per_s": ex2,
                  "compute_source": f"nominal per-SM rates x {sms} SMs x {clk:.0f} MHz"}}


BATCH_METRIC = "batched fwd+bwd ms/iter, 4 scenes x 8 views"
FIT_METRIC = "time to 30 dB PSNR, plain Adam from random init, 512x512 procedural, N=16384"


WARM_METRIC = "time to 30 dB PSNR, learned init vs plain, 512x512 procedural, N=16384"


def main_warmstart(a, torch, dev):
    """--scene warmstart: dataset from the plain loop, network training, and
    wall-clock to 30 dB from the network's proposal vs from random init on
    held-out seeds (value = mean learned seconds; plain and the mean-proposal
    ablation alongside)."""
    from jaxsplat_gb300.warmstart import run_experiment

    res = run_experiment(n_train=a.ws_train_sets, fit_steps=a.ws_fit_steps, epochs=a.ws_epochs,
                         log=lambda m: print(m, file=sys.stderr), device=dev,
                         concurrent=a.ws_concurrent, lr=a.ws_lr)
    ev = res["eval"]
    ok = all(r["learned_reached"] and r["plain_reached"] for r in ev)
    learned = float(np.mean([r["learned_s"] for r in ev]))
    plain = float(np.mean([r["plain_s"] for r in ev]))
    mean = float(np.mean([r["mean_s"] for r in ev]))
    ok_mean = all(r["mean_reached"] for r in ev)
    print(json.dumps({"metric": WARM_METRIC, "value": round(learned, 4) if ok else None,
                      "unit": "s", "plain_value": round(plain, 4) if ok else None,
                      "mean_proposal_value": round(mean, 4) if ok_mean else None,
                      "n_gpus": 1, "steps": len(ev), "warmup": 1, "higher_is_better": False,
                      "scaling": "weak", "vs_baseline": None, "dtype": "bf16 network, f32 render",
                      "data": "synthetic (procedural targets, seeded; training sets fitted here)",
                      "config": {"workload": "warmstart: conv 3-32-64-128-256 + 1x1 head, 32x32x16 "
                                             "Gaussians, 512x512 procedural targets"},
                      "experiment": res}))


NET_METRIC = "warm-start network training step (fwd + bwd + Adam) ms/iter, batch 8, 512x512"


def main_netstep(a, torch, dev):
    """--scene netstep: one training step of the warm-start network (the
    four im2col + tcgen05 GEMM convolutions and the head, the L2 loss, the
    backward with MN-major weight- and data-gradient GEMMs and the fused
    col2im + ReLU gradient, one Adam launch) on seeded random 512x512 images
    and targets resident on the device, batches of 8 cycling through 64."""
    import ctypes as C

    from jaxsplat_gb300 import _lib
    from jaxsplat_gb300.warmstart import IMG, NPARAM, SLOTS, ConvNet, _p

    lib = _lib.load()
    net = ConvNet(dev, seed=a.seed)
    g = torch.Generator(device="cpu").manual_seed(a.seed)
    pool, B = 64, 8
    X = torch.rand(pool, IMG, IMG, 3, generator=g).to(dev).to(torch.bfloat16)
    Y = torch.randn(pool, 32 * 32 * SLOTS * NPARAM, generator=g).to(dev)
    loss = torch.zeros(1, device=dev)

    def step(i):
        idx = torch.arange((i * B) % pool, (i * B) % pool + B, device=dev)
        out = net.forward(X[idx])
        dout = torch.empty_like(out)
        tgt = Y[idx].reshape(-1, SLOTS * NPARAM)
        _lib.check(lib.splat_l2_loss(_p(out), _p(tgt), out.numel(), _p(loss), _p(dout),
                                     C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)),
                   "l2_loss")
        net.backward(dout)
        net.adam(1e-3)

    for i in range(a.warmup):
        step(i)
    net.check()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(a.steps):
        step(a.warmup + i)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    assert int(net.status.item()) == 0, "a tensor-core wait ran out"
    # GEMM FLOPs per step: forward, weight gradients, data gradients (not the
    # first layer's input)
    flops, h = 0, IMG
    for k, L in enumerate(net.layers):
        h = (h - 1) // 2 + 1
        P = B * h * h
        flops += 2 * P * L["k"] * L["cout"] * (2 if k == 0 else 3)
    Hd = net.head
    flops += 3 * 2 * B * 32 * 32 * Hd["k"] * Hd["cout"]
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            bf16_peak = float(json.load(fh)["bf16_tflops"])
    except Exception:
        bf16_peak = None
    tf = flops / (ms * 1e-3) / 1e12
    # libsplat kernels per step: 4 im2col + 14 GEMM + loss + 2 act_grad +
    # 3 col2im_act + 1 Adam
    per_step = 25
    print(json.dumps({"metric": NET_METRIC, "value": round(ms, 4), "unit": "ms",
                      "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
                      "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                      "dtype": "bf16 operands, f32 accumulation", "data": "synthetic (seeded)",
                      "config": {"workload": "warm-start network: conv 3-32-64-128-256 + 1x1 head "
                                             "to 32x32x16x14, batch 8 of 512x512",
                                 "l2": "inputs (64 x 1.5 MB images) cycle through L2"},
                      "gemm_gflop_per_step": round(flops / 1e9, 2),
                      "gemm_tflops": round(tf, 1),
                      "bf16_peak_tflops": bf16_peak,
                      "gpu_launches": per_step * a.steps}))


def main_fit(a, torch, dev):
    """--scene fit: wall-clock of the plain fitting loop (random init, Adam
    lr 1e-2, one CUDA graph per step, PSNR checked every 25 steps) until the
    render reaches 30 dB, on procedural 512x512 targets of held-out seeds."""
    from jaxsplat_gb300.fit import Fitter
    from jaxsplat_gb300.scenes import procedural_target

    seeds = [10_000 + a.seed + k for k in range(max(1, a.steps))]
    runs = []
    for sd in seeds:
        tgt = procedural_target(sd)
        ft = Fitter(tgt, 16384, seed=sd, device=dev)
        ft.run(3)  # warm-up: capture + first steps (untimed)
        ft.check()
        ft = Fitter(tgt, 16384, seed=sd, device=dev)
        ft.capture()
        torch.cuda.synchronize()
        reached, steps, secs, psnr = ft.fit_until(30.0, max_steps=a.fit_max_steps, check_every=25)
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        ft.run(20)
        t1.record()
        torch.cuda.synchronize()
        runs.append({"seed": sd, "reached": reached, "steps": steps, "seconds": round(secs, 4),
                     "psnr": round(psnr, 2), "ms_per_step": round(t0.elapsed_time(t1) / 20, 4)})
    ok = [r["seconds"] for r in runs if r["reached"]]
    value = round(float(np.mean(ok)), 4) if len(ok) == len(runs) else None
    print(json.dumps({"metric": FIT_METRIC, "value": value, "unit": "s", "n_gpus": 1,
                      "steps": len(runs), "warmup": 3, "higher_is_better": False,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                      "data": "synthetic (procedural targets, seeded)",
                      "config": {"workload": "fit: 512x512 procedural target (64 blobs + 3 "
                                             "gratings), 16384 Gaussians, random init, Adam lr 1e-2",
                                 "max_steps": a.fit_max_steps, "check_every": 25},
                      "runs": runs}))


def main_batch(a, torch, world, rank, local, dist, dev):
    """--scene batch: the multi-scene, multi-view workload (one line)."""
    from jaxsplat_gb300.scenes import BATCH_POINTS, BATCH_SIZES

    points = tuple(max(1, int(n * a.batch_scale)) for n in BATCH_POINTS)
    config = {"workload": "batch: 4 scenes (" + ", ".join(str(n) for n in points)
                          + " Gaussians) x 8 views each, image sizes "
                          + "/".join(f"{w}x{h}" for h, w in BATCH_SIZES)
                          + " mixed, fp32, fwd+bwd with per-view L2 loss",
              "scenes": list(points), "views_per_scene": 8,
              "l2": "flushed before every timed step",
              "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}
    if a.impl == "reference":
        if rank != 0:
            return
        from oracle import ref

        if not ref.available():
            print(json.dumps({"impl": "reference", "unavailable":
                              "reference kernels (oracle/_ref) not built on this machine"}))
            return
        st = RefBatchStep(a.seed, dev, points)
    else:
        st = BatchStep(a.seed, dev, graph=not a.no_graph, autotune=a.autotune,
                       log=lambda m: print(m, file=sys.stderr), points=points)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        total = time_device(st, a.steps, a.warmup, flush)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    total = max_over_ranks(total, dist, dev)
    e2e_ms, bi, bo = time_e2e(st, max(3, a.steps // 2), flush)
    e2e_ms = max_over_ranks(e2e_ms, dist, dev)
    if rank != 0:
        dist.destroy_process_group()
        return
    value = whole_job_ms_per_step(total, a.steps, world)
    line = {"metric": BATCH_METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(total / a.steps, 4),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": config,
            "e2e": {"value": round(e2e_ms / world, 4), "unit": UNIT, "h2d_bytes_per_step": bi,
                    "d2h_bytes_per_step": bo, "link_gbs": link_bandwidth(dev)},
            "clocks": clk.summary()}
    if a.impl == "reference":
        line["impl"] = "reference"
        line["reference_kind"] = ("reference CUDA kernels built from its sources (oracle/_ref), "
                                  "one render call per view, same GPU")
        line["gpu_launches"] = None
    else:
        st.sess.check()
        line["gpu_launches"] = st.launches_per_step() * a.steps
        line["cuda_graph"] = st.graph
        line["block_size"], line["chunk"] = st.sess.bw, st.sess.chunk
        if st.tuning:
            line["autotune_ms"] = {f"bw{k[0]}_chunk{k[1]}": round(v, 3) for k, v in st.tuning.items()}
        b = st.sess.batch
        line["entries"], line["tiles"], line["pixels"] = int(b.num_entries), int(b.num_tiles), int(b.num_pixels)
        if world == 1:
            line["e2e_streamed"] = time_e2e_streamed(st, max(10, a.steps), flush)
        add_stages_and_roofline(line, st, a.steps, flush)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scene", default="hd")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-graph", action="store_true", help="eager launches instead of a CUDA graph")
    ap.add_argument("--fit-max-steps", type=int, default=3000)
    ap.add_argument("--batch-scale", type=float, default=1.0,
                    help="batch scene: scale the scenes' Gaussian counts (profiling runs)")
    ap.add_argument("--ws-train-sets", type=int, default=1000)
    ap.add_argument("--ws-fit-steps", type=int, default=300)
    ap.add_argument("--ws-epochs", type=int, default=60)
    ap.add_argument("--ws-lr", type=float, default=3e-3)
    ap.add_argument("--ws-concurrent", type=int, default=16,
                    help="plain fits run at once while generating the training sets")
    ap.add_argument("--autotune", action="store_true",
                    help="batch scene: sweep block size x scheduler chunk before timing")
    a = ap.parse_args()
    assert a.warmup >= 3, "at least 3 warm-up steps"

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    from jaxsplat_gb300.scenes import make_scene

    if a.scene == "batch":
        return main_batch(a, torch, world, rank, local, dist, dev)
    if a.scene == "fit":
        return main_fit(a, torch, dev)
    if a.scene == "warmstart":
        return main_warmstart(a, torch, dev)
    if a.scene == "netstep":
        return main_netstep(a, torch, dev)
    sc = make_scene(a.scene, seed=a.seed)
    config = {"workload": f"{sc.spec.name}: {sc.spec.num_points} Gaussians, "
                          f"{sc.spec.img_shape[1]}x{sc.spec.img_shape[0]}, block 16, fp32, "
                          "fwd+bwd with L2 loss", "scene": sc.spec.name,
              "num_points": sc.spec.num_points, "img_shape": list(sc.spec.img_shape),
              "block_size": sc.spec.block_width, "l2": "flushed before every timed step",
              "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}

    if a.impl == "reference":
        if rank != 0:
            return
        from oracle import ref

        if not ref.available():
            cb = cpu_baseline(sc)
            print(json.dumps({"impl": "reference", "metric": METRIC, "value": cb["value"],
                              "unit": UNIT, "n_gpus": 0, "steps": 1, "warmup": 0,
                              "ms_per_step": cb["value"], "higher_is_better": False,
                              "dtype": "f32", "data": "synthetic", "config": config,
                              "cpu_baseline": cb, "vs_baseline": None,
                              "e2e": {"value": cb["value"], "unit": UNIT,
                                      "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                              "note": "reference kernels not built: CPU restatement"}))
            return
        st = RefStep(sc, dev)
    else:
        st = OursStep(sc, dev, graph=not a.no_graph)

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        total = time_device(st, a.steps, a.warmup, flush)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    total = max_over_ranks(total, dist, dev)
    e2e_ms, bi, bo = time_e2e(st, max(3, a.steps // 2), flush)
    e2e_ms = max_over_ranks(e2e_ms, dist, dev)
    if rank != 0:
        dist.destroy_process_group()
        return
    ms = total / a.steps
    value = whole_job_ms_per_step(total, a.steps, world)
    line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded, benchmark scene distributions)", "config": config,
            "e2e": {"value": round(e2e_ms / world, 4), "unit": UNIT, "h2d_bytes_per_step": bi,
                    "d2h_bytes_per_step": bo, "link_gbs": link_bandwidth(dev)},
            "clocks": clk.summary()}
    if a.impl == "reference":
        line["impl"] = "reference"
        line["reference_kind"] = ("reference CUDA kernels built from its sources (oracle/_ref), "
                                  "stock lib/ops.cu orchestration, same GPU")
        line["cpu_baseline"] = None
        line["gpu_launches"] = None
    else:
        st.sess.check()  # no step overflowed its capacity, no device check fired
        line["gpu_launches"] = st.launches_per_step() * a.steps
        line["cuda_graph"] = st.graph
        if world == 1:
            line["e2e_streamed"] = time_e2e_streamed(st, max(10, a.steps), flush)
        st.pairs = st.sess.count_pairs()  # work counts of the timed step's list
        add_stages_and_roofline(line, st, a.steps, flush)
        add_compute_roofline(line, st)
        if not a.no_cpu_baseline and world == 1:
            line["cpu_baseline"] = cpu_baseline(sc)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
