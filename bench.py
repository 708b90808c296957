"""Benchmark: forward+backward of the render path, 1M Gaussians at 1920x1080.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--scene hd|uhd|small] [--no-cpu-baseline]

One step = project -> count read -> sort/bin -> rasterize forward -> L2 loss
against a target image -> rasterize backward -> project backward, on seeded
synthetic inputs with the benchmark scene's shapes and distributions.

* ``value``: ms per step with inputs resident in HBM, CUDA events on the
  launching stream, L2 flushed (a 256 MiB write) before every timed step and
  excluded from the timing.
* ``e2e``: the same step with the inputs copied from pinned host memory and
  the loss and the five gradient arrays copied back inside the timed region.
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

# DRAM bytes of one raster_bwd_kernel launch on the 1M-Gaussian 1920x1080
# scene, from `ncu --section MemoryWorkloadAnalysis` (profiles/raster_bwd_hd.md);
# None until captured.
NCU_TRAFFIC = {"raster_bwd": None}


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
    """The render path through libsplat's C ABI (jaxsplat_gb300._ops)."""

    def __init__(self, sc, dev):
        import torch

        from jaxsplat_gb300 import _ops

        self.torch, self.ops, self.sc, self.dev = torch, _ops, sc, dev
        self.kw = dict(sc.kwargs, block_width=sc.spec.block_width)
        self.rkw = dict(img_shape=self.kw["img_shape"], block_width=self.kw["block_width"])
        self.host = {k: torch.from_numpy(getattr(sc, k)).pin_memory()
                     for k in ("means3d", "scales", "quats", "colors", "opacities", "viewmat",
                               "background", "target")}
        self.d = {k: v.to(dev) for k, v in self.host.items()}
        n = sc.spec.num_points
        self.zn = torch.zeros(n, 1, device=dev)
        h, w = self.kw["img_shape"]
        self.zalpha = torch.zeros(h, w, 1, device=dev)
        self.count = None
        self.passes = None

    def launches_per_step(self):
        # project_fwd, emit, hist, offsets, passes x onesweep, tile_bins,
        # raster_fwd, l2_loss, raster_bwd, project_bwd
        return 9 + self.passes

    def step(self, ev=None):
        torch, ops, d, kw = self.torch, self.ops, self.d, self.kw
        rec = (lambda name: ev[name].record()) if ev else (lambda name: None)
        n = d["means3d"].shape[0]
        rec("t0")
        p = ops.project_fwd(d["means3d"], d["scales"], d["quats"], d["viewmat"], **kw)
        rec("t1")
        count = ops.read_counts(n, p["cum_tiles_hit"], p["total"], device=self.dev)
        s = ops.sort_and_bin(count, p["xys"], p["depths"], p["radii"], p["cum_tiles_hit"],
                             **self.rkw)
        rec("t2")
        r = ops.rasterize_fwd(count, s["gaussian_ids_sorted"], s["tile_bins"], p["xys"],
                              p["conics"], d["colors"], d["opacities"], d["background"],
                              **self.rkw)
        rec("t3")
        loss, v_img = ops.l2_loss(r["img"], d["target"])
        rec("t4")
        rb = ops.rasterize_bwd(count, s["gaussian_ids_sorted"], s["tile_bins"], p["xys"],
                               p["conics"], d["colors"], d["opacities"], d["background"],
                               r["final_Ts"], r["final_idx"], v_img, self.zalpha, **self.rkw)
        rec("t5")
        pb = ops.project_bwd(d["means3d"], d["scales"], d["quats"], d["viewmat"], p["cov3d"],
                             p["radii"], p["conics"], p["compensation"], rb["v_xy"], self.zn,
                             rb["v_conic"], self.zn, **kw)
        rec("t6")
        self.count = count
        if self.passes is None:
            tx = (kw["img_shape"][1] + kw["block_width"] - 1) // kw["block_width"]
            ty = (kw["img_shape"][0] + kw["block_width"] - 1) // kw["block_width"]
            t = tx * ty
            end_bit = 32 + t.bit_length() + 1
            self.passes = (end_bit + 7) // 8
        return loss, [pb["v_mean3d"], pb["v_scale"], pb["v_quat"], rb["v_colors"],
                      rb["v_opacity"]]

    def upload(self):
        for k, v in self.host.items():
            self.d[k].copy_(v, non_blocking=True)


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


# ---------------------------------------------------------------------------

def time_device(st, steps, warmup, flush, stage_events=False):
    """Per-step CUDA-event timing, L2 flushed before each step (untimed)."""
    torch = st.torch
    for _ in range(warmup):
        st.step()
    torch.cuda.synchronize()
    total = 0.0
    stages = {}
    names = ["t0", "t1", "t2", "t3", "t4", "t5", "t6"]
    for _ in range(steps):
        flush.fill_(1)
        ev = {k: torch.cuda.Event(enable_timing=True) for k in names} if stage_events else None
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        st.step(ev)
        b.record()
        torch.cuda.synchronize()
        total += a.elapsed_time(b)
        if ev:
            for (x, y), nm in zip(zip(names, names[1:]), ["project_fwd", "count+sort", "raster_fwd",
                                                          "l2_loss", "raster_bwd", "project_bwd"]):
                stages[nm] = stages.get(nm, 0.0) + ev[x].elapsed_time(ev[y])
    return total, stages


def time_e2e(st, steps, flush):
    """Host buffers: H2D of the inputs and D2H of loss + gradients inside."""
    torch = st.torch
    out_host = None
    total = 0.0
    bi = sum(v.numel() * v.element_size() for v in st.host.values())
    bo = 0
    for _ in range(steps):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        st.upload()
        loss, grads = st.step()
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scene", default="hd")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
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
        st = OursStep(sc, dev)

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        total, stages = time_device(st, a.steps, a.warmup, flush, stage_events=a.impl == "ours")
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if dist:
        t = torch.tensor([total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = float(t.item())
    e2e_ms, bi, bo = time_e2e(st, max(3, a.steps // 2), flush)
    if dist:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    if rank != 0:
        dist.destroy_process_group()
        return
    ms = total / a.steps
    value = ms / world
    line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded, benchmark scene distributions)", "config": config,
            "e2e": {"value": round(e2e_ms / world, 4), "unit": UNIT, "h2d_bytes_per_step": bi,
                    "d2h_bytes_per_step": bo},
            "clocks": clk.summary()}
    if a.impl == "reference":
        line["impl"] = "reference"
        line["reference_kind"] = ("reference CUDA kernels built from its sources (oracle/_ref), "
                                  "stock lib/ops.cu orchestration, same GPU")
        line["cpu_baseline"] = None
        line["gpu_launches"] = None
    else:
        line["gpu_launches"] = st.launches_per_step() * a.steps
        count = st.count
        h, w = sc.spec.img_shape
        P = h * w
        stage_ms = {k: v / a.steps for k, v in stages.items()}
        line["stages_ms"] = {k: round(v, 4) for k, v in stage_ms.items()}
        line["num_intersects"] = count
        dominant = max(stage_ms, key=stage_ms.get)
        # algorithmic bytes per launch ("Roofline"): raster
        # backward reads 40 B per intersection (id + xy + opacity + conic +
        # color) and issues 9 fp32 atomics (36 B) per (tile, Gaussian) pair,
        # and reads 24 B per pixel (final_Ts, final_idx, v_img, v_img_alpha).
        bytes_by_stage = {"raster_bwd": 76 * count + 24 * P,
                          "raster_fwd": 40 * count + 20 * P,
                          "count+sort": 24 * count * st.passes + 40 * count,
                          "project_fwd": 100 * sc.spec.num_points,
                          "project_bwd": 140 * sc.spec.num_points,
                          "l2_loss": 36 * P}
        peak, src = _peaks()
        achieved = bytes_by_stage[dominant] / (stage_ms[dominant] * 1e-3) / 1e9
        traffic = NCU_TRAFFIC.get(dominant)
        line["roofline"] = {"kernel": dominant, "bound": "hbm", "achieved": round(achieved, 1),
                            "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                            "peak_source": src, "traffic": traffic,
                            "algorithmic_bytes": bytes_by_stage[dominant]}
        if not a.no_cpu_baseline and world == 1:
            line["cpu_baseline"] = cpu_baseline(sc)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
