"""Benchmark: Msamples/s of the Eleven Renderer sample path at 1080p on GB300.

Workload (default): the full-feature scene -- 1920x1080, max depth 8,
~1.18M triangles in 200 seeded displaced spheres, ten 512^2 value-noise
baseColor textures, a 2048x1024 log-normal HDR environment with a sun patch,
4 point lights, thin-lens camera (aperture 0.05, focus 10), MIS over all
strategies.  Seeded synthetic data stands in for the reference's scenes.

A step is one sample per pixel of the 1080p frame (2,073,600 path samples)
through the wavefront tracer.  `value` is device-timed with CUDA events on
the render stream, scene resident in HBM; `e2e` goes through the C-ABI call
a user makes (er_render with host output buffers, the image read back every
step).  The working set (BVH + triangles + textures + environment, ~0.2 GB,
plus ~0.6 GB of queue traffic per step) exceeds the 126 MB L2, so no flush
is inserted between steps.

--impl reference times the reference's CPU path on the host cores: the
oracle port of the reference (its depth-18 BVH, traversal and shading,
restated in C), all host threads, a bounded pixel subset per step.  Its
line also carries `reference_cuda`: the reference's own CUDA renderer
(kernel.cu, built for sm_103a from the reference tree with four textual
patches) timed on the GPU for this config and for the small scene.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tfg-pathtracer_gb300"))

import numpy as np  # noqa: E402

METRIC = "Msamples/s at 1080p (plain wavefront, max depth 8)"
UNIT = "Msamples/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=128)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c1", choices=["c1", "c0", "c2", "c4"])
    ap.add_argument("--fd-params", type=int, default=32, help="c4: parameters in the finite-difference check")
    ap.add_argument("--jobs", type=int, default=64, help="c2: number of batch jobs")
    ap.add_argument("--steady", action="store_true",
                    help="c2: also time every job alone at full-size waves (its steady-state cost per sample) "
                         "and print the sum beside the plain and batched times")
    ap.add_argument("--bvh", default="fp32", choices=["fp32", "q8"])
    ap.add_argument("--max-leaf", type=int, default=0, help="triangles per BVH leaf (0 = library default)")
    ap.add_argument("--builder", default="host", choices=["host", "gpu"], help="BVH builder")
    ap.add_argument("--env-sampling", default="search", choices=["search", "alias"],
                    help="HDRI light sampling: the reference's CDF search or the alias table")
    ap.add_argument("--e2e-steps", type=int, default=16)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sub", action="store_true",
                    help="c1: skip the batched (64-job) and adjoint sub-records of the default line")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="--impl reference: skip timing the reference's CUDA renderer on the GPU")
    ap.add_argument("--launch-rays", type=int, default=-1,
                    help="print the rays traced by trace launch B of a 1-spp wave (extension rays of bounce B "
                         "+ shadow rays of bounce B-1) and exit; used to turn an ncu capture of that launch "
                         "into DRAM bytes per ray")
    return ap.parse_args()


def make_scene(cfg):
    from eleven import scenes
    if cfg == "c0":
        return scenes.config0(), 4, dict(workload="c0: 320x240 pinhole, 20,482 tris, 1 point light, constant env",
                                         resolution="320x240", max_depth=4)
    return scenes.config1(), 8, dict(
        workload="c1: 1920x1080 thin lens, ~1.18M tris (200 displaced spheres), 10 textures 512^2, "
                 "2048x1024 HDR env + sun, 4 point lights",
        resolution="1920x1080", max_depth=8)


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        pg = dist
    return rank, world, local, pg


def barrier_max(pg, local, value):
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=f"cuda:{local}")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg, local):
    if pg is not None:
        import torch
        pg.barrier()
        torch.cuda.synchronize(local)


class Clocks:
    """nvidia-smi sampling during the timed region (200 ms)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def host_buffers(npix):
    """Film readback buffers in page-locked host memory (torch's pinned
    allocator), else pageable numpy arrays; returns the kind as well."""
    try:
        import torch
        if torch.cuda.is_available():
            b = torch.empty((npix, 4), dtype=torch.float32, pin_memory=True)
            s = torch.empty((npix,), dtype=torch.int32, pin_memory=True)
            c = torch.empty((npix,), dtype=torch.int32, pin_memory=True)
            return b.numpy(), s.numpy().view(np.uint32), c.numpy().view(np.uint32), "pinned"
    except Exception:
        pass
    return (np.zeros((npix, 4), np.float32), np.zeros(npix, np.uint32), np.zeros(npix, np.uint32), "pageable")


def traffic_per_ray():
    """DRAM bytes per traced ray of the dominant kernel from the committed ncu
    summary (profiles/extend_c1_dram.json), or None."""
    p = os.path.join(ROOT, "profiles", "extend_c1_dram.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


def l2_roofline(config, rays, trace_launches, trace_ms, hits, shade_ms, shade_launches, device):
    """L2 and DRAM bytes of k_trace / k_shade per ray / per hit from the
    committed ncu capture (profiles/l2_dram_c1.json), scaled to the live
    launches, against this GPU's L2 read ceiling measured by the library."""
    from eleven import _abi as A
    from eleven import _lib
    try:
        l2_peak = _lib.device_bandwidth(A.ER_BW_L2_READ, 64 << 20, 40, device)
        hbm_own = _lib.device_bandwidth(A.ER_BW_HBM_COPY, 1 << 30, 4, device)
    except Exception as e:  # noqa: BLE001
        return {"l2": {"unavailable": str(e)}}
    p = os.path.join(ROOT, "profiles", "l2_dram_c1.json")
    prof = json.load(open(p)) if os.path.exists(p) else None
    res = {"peak_l2_read": round(l2_peak, 1), "peak_hbm_copy_own_kernel": round(hbm_own, 1), "unit": "GB/s",
           "peak_source": "er_device_bandwidth on this GPU (64 MiB L2-resident read x40; 1 GiB copy x4)"}
    if prof and prof.get("config") == config:
        t, sh = prof["k_trace"], prof["k_shade"]
        tl = trace_ms * 1e-3 / max(trace_launches, 1)
        per_launch = rays / max(trace_launches, 1)
        res["k_trace"] = {"l2_bytes_per_ray": round(t["lts_bytes"] / t["rays"], 1),
                          "achieved_l2": round(t["lts_bytes"] / t["rays"] * per_launch / tl / 1e9, 1),
                          "dram_bytes_per_ray": round(t["dram_bytes"] / t["rays"], 1),
                          "achieved_dram": round(t["dram_bytes"] / t["rays"] * per_launch / tl / 1e9, 1)}
        res["k_trace"]["frac_l2"] = round(res["k_trace"]["achieved_l2"] / l2_peak, 4)
        sl = shade_ms * 1e-3 / max(shade_launches, 1)
        hp = hits / max(shade_launches, 1)
        res["k_shade"] = {"l2_bytes_per_hit": round(sh["lts_bytes"] / sh["hits"], 1),
                          "achieved_l2": round(sh["lts_bytes"] / sh["hits"] * hp / sl / 1e9, 1),
                          "dram_bytes_per_hit": round(sh["dram_bytes"] / sh["hits"], 1),
                          "achieved_dram": round(sh["dram_bytes"] / sh["hits"] * hp / sl / 1e9, 1)}
        res["k_shade"]["frac_l2"] = round(res["k_shade"]["achieved_l2"] / l2_peak, 4)
        for k in ("issue_active", "simt_efficiency"):
            if k in t:
                res["k_trace"][k] = t[k]
            if k in sh:
                res["k_shade"][k] = sh[k]
        res["source"] = "profiles/l2_dram_c1.json (" + prof.get("command", "") + ")"
    return {"l2": res}


def roofline_of(kname, achieved, peak, peak_src, traffic, b_ray, nl, kms, prof_steps, l2, rays, device, clk):
    """The dominant kernel's roofline.  k_trace is bound by SM issue (and the
    load latency behind it), not by a memory: its bytes mostly come from L2
    and it moves a fifth of the L2 ceiling.  So the headline fraction is
    warp instructions issued per second against the schedulers' issue rate
    (4 per SM per cycle at the SM clock), with warp instructions per ray from
    the committed ncu capture and the live launch times; the HBM figure
    (algorithmic bytes over the copy bandwidth) and the L2 figure ride
    along.  Without the capture the HBM figure is the headline."""
    hbm = {"achieved": round(achieved, 1), "peak": peak, "peak_source": peak_src, "unit": "GB/s",
           "frac": round(achieved / peak, 4), "traffic": traffic, "algorithmic_bytes_per_ray": round(b_ray, 1),
           "note": "algorithmic bytes (32 + 16 + 32 box tests + 36 triangle tests per ray) over the copy bandwidth; "
                   "DRAM carries `traffic` of them, the rest comes from L2"}
    common = {"kernel": kname, "launches": int(nl), "avg_launch_ms": round(kms / max(nl, 1), 4),
              "timing": f"CUDA events after every launch, profiled pass of {prof_steps} steps on one stream"}
    p = os.path.join(ROOT, "profiles", "l2_dram_c1.json")
    prof = json.load(open(p)) if os.path.exists(p) else None
    try:
        import torch
        sms = torch.cuda.get_device_properties(device).multi_processor_count
    except Exception:  # noqa: BLE001
        sms = None
    mhz = (clk or {}).get("sm_max_mhz")
    if not mhz:
        pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
        mhz = json.load(open(pp)).get("sm_max_mhz") if os.path.exists(pp) else None
    if prof and "k_trace" in prof and sms and mhz:
        t = prof["k_trace"]
        per_ray = t["warp_inst"] / t["rays"]
        inst_s = per_ray * rays / max(nl, 1) / (kms * 1e-3 / max(nl, 1)) / 1e9
        peak_issue = 4 * sms * mhz * 1e6 / 1e9
        return {"bound": "issue", **common, "achieved": round(inst_s, 1), "peak": round(peak_issue, 1),
                "unit": "G warp instructions/s", "frac": round(inst_s / peak_issue, 4), "traffic": traffic,
                "peak_source": f"4 issue slots x {sms} SMs x {mhz:.0f} MHz (max SM clock)",
                "warp_inst_per_ray": round(per_ray, 1), "simt_efficiency": t.get("simt_efficiency"),
                "hbm": hbm, **l2}
    return {"bound": "hbm", **common, **{k: v for k, v in hbm.items() if k != "note"}, **l2}


def cpu_baseline(arrays, max_depth, seconds, seed=0):
    """Oracle port of the reference on all host threads, bounded pixel subset."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    W, H = arrays.camera["x_res"], arrays.camera["y_res"]
    orc = O.OrcScene(arrays)
    cores = os.cpu_count() or 1
    # rate probe, grown until it is long enough to time (thread start-up
    # dominates a few pixels)
    stride, spp = 4096, 1
    while True:
        t = time.perf_counter()
        orc.render(spp=spp, max_depth=max_depth, seed=seed, pixel_stride=stride)
        dt = max(time.perf_counter() - t, 1e-3)
        if dt >= 0.2 or spp >= 4096:
            break
        if stride > 1:
            stride = max(1, stride // 8)
        else:
            spp *= 8
    rate = ((W * H + stride - 1) // stride) * spp / dt
    # a pixel subset of large frames; several samples of every pixel of
    # small ones, so that the sample is about `seconds` of work either way
    stride = max(1, int(W * H / max(1.0, rate * seconds)))
    spp = max(1, int(rate * seconds / (W * H))) if stride == 1 else 1
    n = (W * H + stride - 1) // stride * spp
    t = time.perf_counter()
    r = orc.render(spp=spp, max_depth=max_depth, seed=seed, pixel_stride=stride)
    dt = time.perf_counter() - t
    orc.close()
    return dict(value=n / dt / 1e6, unit=UNIT, cores=cores, kind="port",
                sample=f"{spp} spp on every {stride}th pixel of the {W}x{H} frame ({n} samples, {dt:.1f} s, "
                       f"{int(r['pathcount'].sum())} path vertices)"), dt


REF_CUDA_PATCHES = [
    "kernel.cu:156,158 `#if USEBVH:` / `#else:` without the colon (MSVC-only preprocessor syntax)",
    "kernel.cu:781,783 std::sinf / std::cosf -> sinf / cosf (host debug printer; not in libstdc++'s std)",
    "Definitions.h:9 MAXBOUNCES settable per build (4 for c0, 8 for c1)",
    "kernel.cu:185 point-light index (int)(n * r1) clamped to n - 1 (cuRAND's uniform may return 1)",
]


def reference_cuda(arrays, max_depth, warm, spp):
    """The reference's own CUDA renderer (kernel.cu renderingKernel, one
    launch per sample) on this GPU through oracle/ref_cuda_main.cpp, built
    from the reference tree by `make -C oracle refcuda` with the patches
    above; CUDA events on the reference's kernelStream around renderCuda."""
    from eleven.build import ORACLE, REF_SRC
    if not os.path.isdir(REF_SRC):
        return {"unavailable": "reference sources not present"}
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no CUDA device visible"}
    except ImportError:
        pass
    t = time.perf_counter()
    r = subprocess.run(["make", "-s", "-C", ORACLE, "-j4", "refcuda", "REF_DIR=" + REF_SRC], capture_output=True,
                       text=True)
    if r.returncode != 0:
        return {"unavailable": "reference CUDA build failed: " + (r.stdout + r.stderr)[-300:]}
    build_s = time.perf_counter() - t
    sys.path.insert(0, ORACLE)
    import refcuda_scene
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, "scene.ersc")
        refcuda_scene.write(arrays, f)
        exe = os.path.join(ORACLE, "_ref", f"ref_cuda_d{max_depth}")
        if not os.path.exists(exe):
            return {"unavailable": f"no reference build for depth {max_depth}"}
        r = subprocess.run([exe, f, str(warm), str(spp)], capture_output=True, text=True, timeout=1200)
    if r.returncode != 0:
        return {"unavailable": f"reference CUDA run exited {r.returncode}: " + r.stdout[-200:] + r.stderr[-200:]}
    res = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    W, H = res["width"], res["height"]
    return {"value": round(W * H * spp / res["ms"] / 1e3, 3), "unit": UNIT, "ms": round(res["ms"], 2),
            "spp": spp, "warmup_spp": warm, "resolution": f"{W}x{H}", "max_bounces": res["max_bounces"],
            "kpaths_per_s": round(res["path_vertices"] / res["ms"], 1),
            "render_setup_s": round(res["render_setup_ms"] / 1e3, 2), "build_s": round(build_s, 1),
            "timing": "CUDA events on the reference's kernelStream around renderCuda (one renderingKernel "
                      "launch and one stream synchronisation per sample, kernel.cu:665-686)",
            "nvcc": "-O3 -use_fast_math -rdc=true -lineinfo, sm_103a (tfg-pathtracer.vcxproj:139-141)",
            "patches": REF_CUDA_PATCHES}


def run_reference(args):
    rank, world, local, pg = dist_setup(args.gpus)
    if rank != 0:
        return 0
    arrays, max_depth, cfg = make_scene(args.config)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    W, H = arrays.camera["x_res"], arrays.camera["y_res"]
    orc = O.OrcScene(arrays)
    cores = os.cpu_count() or 1
    # size one step to ~0.5 s of host work (the default 128 steps then take about a minute)
    t = time.perf_counter()
    orc.render(spp=1, max_depth=max_depth, pixel_stride=4096)
    rate = ((W * H + 4095) // 4096) / max(time.perf_counter() - t, 1e-3)
    stride = max(1, int(W * H / max(1.0, rate * 0.5)))
    n = (W * H + stride - 1) // stride
    for i in range(args.warmup):
        orc.render(spp=1, max_depth=max_depth, sample_begin=i, pixel_stride=stride)
    t = time.perf_counter()
    for i in range(args.steps):
        orc.render(spp=1, max_depth=max_depth, sample_begin=args.warmup + i, pixel_stride=stride)
    dt = time.perf_counter() - t
    value = args.steps * n / dt / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, reference scene shapes)", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"per step 1 spp on every {stride}th pixel ({n} samples)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    orc.close()
    if not args.no_reference_cuda:
        # the reference's CUDA renderer on this GPU: this config, and the
        # small scene at its stated 16 spp x 4
        rc = {args.config: reference_cuda(arrays, max_depth, 1, 4 if args.config == "c1" else 64)}
        if args.config != "c0":
            a0, d0, _ = make_scene("c0")
            rc["c0"] = reference_cuda(a0, d0, 16, 64)
        line["reference_cuda"] = rc
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    from eleven import _abi as A
    from eleven import _lib
    rank, world, local, pg = dist_setup(args.gpus)
    arrays, max_depth, cfg = make_scene(args.config)
    W, H = arrays.camera["x_res"], arrays.camera["y_res"]
    npix = W * H
    fmt = A.ER_BVH_Q8 if args.bvh == "q8" else A.ER_BVH_FP32
    builder = A.ER_BUILDER_GPU if args.builder == "gpu" else A.ER_BUILDER_HOST
    scene = _lib.Scene(arrays, bvh_format=fmt, max_leaf=args.max_leaf, device=local, builder=builder)
    info = scene.info()
    base = rank * (args.warmup + args.steps + args.e2e_steps + 8)

    # calibration (untimed): node visits / triangle tests per ray
    cal = scene.render(spp=1, max_depth=max_depth, sample_begin=base,
                       flags=A.ER_RENDER_COUNT | A.ER_RENDER_NO_OUTPUT)["stats"]
    n_box_c = 4.0 * cal.closest_nodes / max(cal.rays_closest, 1)
    n_tri_c = cal.closest_tris / max(cal.rays_closest, 1)
    n_box_s = 4.0 * cal.shadow_nodes / max(cal.rays_shadow, 1)
    n_tri_s = cal.shadow_tris / max(cal.rays_shadow, 1)
    b_ray_c = 32 + 16 + 32 * n_box_c + 36 * n_tri_c
    b_ray_s = 32 + 16 + 32 * n_box_s + 36 * n_tri_s

    env_flag = A.ER_RENDER_ENV_ALIAS if args.env_sampling == "alias" else 0
    scene.render(spp=args.warmup, max_depth=max_depth, sample_begin=base + 1, flags=A.ER_RENDER_NO_OUTPUT | env_flag)
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    barrier(pg, local)
    t0 = time.perf_counter()
    st = scene.render(spp=args.steps, max_depth=max_depth, sample_begin=base + 1 + args.warmup,
                      flags=A.ER_RENDER_NO_OUTPUT | env_flag)["stats"]
    wall = time.perf_counter() - t0
    ms = barrier_max(pg, local, st.ms)
    clk = clocks.stop()
    value = world * args.steps * npix / ms / 1e3
    # per-kernel times: a profiled pass (events after every launch, waves on
    # one stream) of the same samples
    prof_steps = min(args.steps, 8)
    pst = scene.render(spp=prof_steps, max_depth=max_depth, sample_begin=base + 1 + args.warmup,
                       flags=A.ER_RENDER_NO_OUTPUT | A.ER_RENDER_PROFILE | env_flag)["stats"]

    # the timing rule's L2 statement: no flush between steps; the scene is
    # larger than L2 (c1) or L2-resident (c0), and the path state of every
    # wave streams through HBM either way
    scene_mb = info.device_bytes / 1e6
    l2_note = (f"no flush: scene {scene_mb:.0f} MB " + ("> 126 MB L2" if scene_mb > 126 else "(L2-resident)") +
               ", path state streamed through HBM")
    # e2e through the C-ABI with host buffers (page-locked, as a caller
    # that reads the film every step allocates them), one 1-spp call per step
    beauty, samples, pathcount, host_mem = host_buffers(npix)
    import ctypes as C
    L = _lib.load()
    o = A.er_render_opts(1, 0, max_depth, 0, 0, 0, 0)
    barrier(pg, local)
    t0 = time.perf_counter()
    for i in range(args.e2e_steps):
        o.sample_begin = base + 2 + args.warmup + args.steps + i
        o.flags = (A.ER_RENDER_CONTINUE if i else 0) | env_flag
        _lib.check(L.er_render(scene.h, C.byref(o), beauty.ctypes.data_as(C.c_void_p), None, None, None,
                               samples.ctypes.data_as(C.c_void_p), pathcount.ctypes.data_as(C.c_void_p), None),
                   "er_render")
    e2e_s = barrier_max(pg, local, time.perf_counter() - t0)
    e2e = world * args.e2e_steps * npix / e2e_s / 1e6
    d2h = beauty.nbytes + samples.nbytes + pathcount.nbytes

    # roofline of the dominant kernel: k_trace (extension + shadow rays)
    kname, kms, nl = "k_trace", pst.stage_ms[1], pst.stage_launches[1]
    rays = pst.rays_closest + pst.rays_shadow
    alg_bytes = pst.rays_closest * b_ray_c + pst.rays_shadow * b_ray_s
    b_ray = alg_bytes / max(rays, 1)
    peak, peak_src = peaks()
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    tr = traffic_per_ray()
    traffic = None
    if tr and tr.get("kernel") == kname and args.config == tr.get("config"):
        traffic = tr["dram_bytes_per_ray"] * rays / max(nl, 1)
    stage = {n: round(pst.stage_ms[k] / prof_steps, 3) for k, n in enumerate(A.STAGES)}
    # L2 side of the same kernels: L2 bytes (lts__t_bytes) per ray / per hit
    # from one ncu capture each, over the live launch times, against the L2
    # read ceiling the library measures on this GPU (er_device_bandwidth)
    l2 = l2_roofline(args.config, rays, nl, kms, pst.path_vertices, pst.stage_ms[2], pst.stage_launches[2], local)

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, reference scene shapes)",
        "config": dict(cfg, spp_per_step=1, bvh=args.bvh, max_leaf_tris=args.max_leaf or 4, bvh_builder=args.builder,
                       env_sampling=args.env_sampling,
                       triangles=arrays.tri_count,
                       l2=l2_note, parallelism="replicas" if world > 1 else "1 GPU"),
        "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": int(C.sizeof(A.er_render_opts)),
                "d2h_bytes_per_step": int(d2h), "host_memory": host_mem},
        "gpu_launches": int(st.kernel_launches),
        "roofline": roofline_of(kname, achieved, peak, peak_src, traffic, b_ray, nl, kms, prof_steps, l2, rays,
                                local, clk),
        "rays_per_s": {"closest": round(st.rays_closest / ms / 1e3, 1), "shadow": round(st.rays_shadow / ms / 1e3, 1),
                       "unit": "Mrays/s"},
        "path_vertices_per_s": round(st.path_vertices / ms / 1e3, 1),
        "stage_ms_per_step": stage,
        "profiled_ms_per_step": round(pst.ms / prof_steps, 4),
        "per_ray": {"closest_box_tests": round(n_box_c, 2), "closest_tri_tests": round(n_tri_c, 2),
                    "shadow_box_tests": round(n_box_s, 2), "shadow_tri_tests": round(n_tri_s, 2)},
        "scene": {"bvh_build_ms": round(info.bvh_build_ms, 1), "upload_ms": round(info.upload_ms, 1),
                  "nodes": int(info.node_count), "device_bytes": int(info.device_bytes)},
        "wall_s_timed": round(wall, 3),
    }
    if clk:
        line["clocks"] = clk
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb, _ = cpu_baseline(arrays, max_depth, args.cpu_seconds)
        line["cpu_baseline"] = cb
    scene.close()
    if rank == 0 and world == 1 and args.config == "c1" and not args.no_sub:
        # the other two parts of the headline metric, measured in the same
        # run: the batched 8-bit-BVH form against the plain tracer on the
        # 64-job workload, and adjoint full-gradient evaluations per second
        b = measure_batch(args.jobs, 2, 1)
        line["batched"] = {k: b[k] for k in ("metric", "value", "unit", "steps", "ms_per_step", "config", "plain",
                                              "batched", "speedup_batched_vs_plain", "films_bit_identical", "clocks")
                           if k in b}
        a = measure_adjoint(3, 1, args.fd_params)
        line["adjoint"] = {k: a[k] for k in ("metric", "value", "unit", "ms_per_step", "config", "forward_ms",
                                             "backward_ms", "backward_msamples_per_s", "fd_check", "gpu_launches",
                                             "clocks")
                           if k in a}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


def run_batch(args):
    line = measure_batch(args.jobs, args.steps, args.warmup)
    if args.steady:
        line["steady"] = measure_steady(args.jobs)
    print(json.dumps(line), flush=True)
    return 0


def measure_steady(n_jobs):
    """The 64-job workload's cost if every job ran at the efficiency of a
    large render of its own scene: each job alone with 4 full-size waves
    (4 x floor(2^24 / pixels) samples per pixel), its time scaled to the
    job's own sample count, summed over the jobs (FP32 and 8-bit nodes).
    Batching removes small-job and launch losses; it cannot go below this
    sum unless jobs gain from sharing waves."""
    from eleven import _abi as A
    from eleven import _lib, scenes
    arrays, jobs = scenes.config2(n_jobs=n_jobs)
    NO = A.ER_RENDER_NO_OUTPUT
    tot = {"samples": 0, "fp32_ms": 0.0, "q8_ms": 0.0}
    small = []
    for a, j in zip(arrays, jobs):
        npix = a.camera["x_res"] * a.camera["y_res"]
        spp_s = 4 * max(1, (1 << 24) // npix)
        samples = j["spp"] * npix
        for fmt, key in ((A.ER_BVH_FP32, "fp32_ms"), (A.ER_BVH_Q8, "q8_ms")):
            s = _lib.Scene(a, bvh_format=fmt)  # one scene at a time: full-size waves hold ~10 GB each
            # the first render allocates the waves (inside its timed span): untimed
            s.render(spp_s, max_depth=j["max_depth"], seed=j["seed"] + 2, flags=NO)
            ms = s.render(spp_s, max_depth=j["max_depth"], seed=j["seed"] + 1, flags=NO)["stats"].ms
            s.close()
            tot[key] += ms * samples / (spp_s * npix)
        tot["samples"] += samples
    return {"what": "sum over jobs of each job's cost per sample alone at 4 full-size waves x its samples",
            "fp32_ms": round(tot["fp32_ms"], 2), "q8_ms": round(tot["q8_ms"], 2),
            "fp32_msamples_per_s": round(tot["samples"] / tot["fp32_ms"] / 1e3, 1),
            "q8_msamples_per_s": round(tot["samples"] / tot["q8_ms"] / 1e3, 1)}


def measure_batch(n_jobs, steps, warmup):
    """c2: 64 heterogeneous scenes/views.  Plain = each job through er_render
    on its own scene, one after another (FP32 BVH); batched = all jobs in one
    er_batch (8-bit BVH, autotuned schedule, one CUDA graph per render).  A
    step renders every job once; both forms give the same films bit for
    bit (checked here on a few jobs), so the image error is equal."""
    from eleven import _abi as A
    from eleven import _lib, scenes
    t_gen = time.perf_counter()
    arrays, jobs = scenes.config2(n_jobs=n_jobs)
    t_gen = time.perf_counter() - t_gen
    t_build = time.perf_counter()
    plain = [_lib.Scene(a) for a in arrays]
    q8 = [_lib.Scene(a, bvh_format=A.ER_BVH_Q8) for a in arrays]
    t_build = time.perf_counter() - t_build
    samples = sum(j["spp"] * a.camera["x_res"] * a.camera["y_res"] for a, j in zip(arrays, jobs))

    def plain_pass(flags=A.ER_RENDER_NO_OUTPUT):
        ms = 0.0
        for s, j in zip(plain, jobs):
            ms += s.render(j["spp"], max_depth=j["max_depth"], seed=j["seed"], flags=flags)["stats"].ms
        return ms

    for _ in range(max(1, warmup)):
        plain_pass()
    clocks = Clocks(0)
    clocks.start()
    time.sleep(0.3)
    t0 = time.perf_counter()
    plain_ms = [plain_pass() for _ in range(steps)]
    plain_wall = (time.perf_counter() - t0) / steps

    b = _lib.Batch(q8, bvh_format=A.ER_BVH_Q8)
    b.set_jobs(jobs)
    t_tune = time.perf_counter()
    tuning = b.autotune(reps=1)
    t_tune = time.perf_counter() - t_tune
    for _ in range(max(1, warmup)):
        b.render()
    t0 = time.perf_counter()
    stats = [b.render() for _ in range(steps)]
    batch_wall = (time.perf_counter() - t0) / steps
    clk = clocks.stop()
    batch_ms = [s.ms for s in stats]
    # same films: compare a few jobs with the plain renders (host output)
    same = True
    for k in range(0, len(jobs), max(1, len(jobs) // 4)):
        j = jobs[k]
        ref = plain[k].render(j["spp"], max_depth=j["max_depth"], seed=j["seed"])["beauty"]
        same &= bool(np.array_equal(ref.view(np.uint32), b.read(k)["beauty"].view(np.uint32)))
    n_waves, batch_bytes = b.info()
    pm, bm = float(np.median(plain_ms)), float(np.median(batch_ms))
    line = {
        "metric": "Msamples/s, 64-job batch (batched 8-bit BVH vs plain sequential)", "value": round(samples / bm / 1e3, 3),
        "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": round(bm, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, reference scene shapes)",
        "config": {"workload": f"c2: {len(jobs)} jobs, resolutions 128^2..1024x768, spp 4/16/64, depth 4-8, "
                               "10k-500k tris each (displaced spheres), 1-4 lights, 512x256 HDR env",
                   "samples_per_step": int(samples), "triangles": int(sum(a.tri_count for a in arrays)),
                   "l2": "working set > 126 MB L2 (no flush)"},
        "plain": {"value": round(samples / pm / 1e3, 3), "ms_per_step": round(pm, 3),
                  "wall_ms_per_step": round(plain_wall * 1e3, 3), "bvh": "fp32",
                  "launches_per_step": None},
        "batched": {"value": round(samples / bm / 1e3, 3), "ms_per_step": round(bm, 3),
                    "wall_ms_per_step": round(batch_wall * 1e3, 3), "bvh": "q8",
                    "gpu_launches": int(stats[-1].kernel_launches), "waves": n_waves,
                    "tuning": {"wave_paths": tuning.wave_paths, "trace_blocks_per_sm": tuning.trace_blocks_per_sm,
                               "shade_blocks_per_sm": tuning.shade_blocks_per_sm,
                               "split_trace": tuning.split_trace, "one_stream": tuning.one_stream},
                    "autotune_s": round(t_tune, 1), "device_bytes": batch_bytes},
        "speedup_batched_vs_plain": round(pm / bm, 3),
        "films_bit_identical": same,
        "setup_s": {"generate": round(t_gen, 1), "scenes": round(t_build, 1)},
    }
    if clk:
        line["clocks"] = clk
    b.close()
    for s in plain + q8:
        s.close()
    return line


def run_adjoint(args):
    line = measure_adjoint(args.steps, args.warmup, args.fd_params)
    print(json.dumps(line), flush=True)
    return 0


def measure_adjoint(steps, warmup, fd_params):
    """c4: gradients of an L2 image loss with respect to 98,624 parameters
    (64 objects x 5 Disney parameters + a 256x128 RGB environment), 512x512,
    64 spp forward + 64 spp path-replay adjoint, max depth 6.  A step is one
    forward render (er_render) plus one er_backward; value = full-gradient
    evaluations per second.  The check: central differences (h = 1e-3,
    common random numbers) of the detached estimator on --fd-params random
    differentiable parameters, at 256 spp, from the films' FP64 sums."""
    from eleven import _abi as A
    from eleven import _lib, scenes
    spp, depth = 64, 6
    arrays = scenes.config4()
    target = scenes.config4(param_seed=41)
    s = _lib.Scene(arrays)
    t = _lib.Scene(target)
    T = t.render(spp, max_depth=depth, seed=99)["beauty"]
    t.close()
    m0, e0 = s.get_params()
    n_params = m0.size + e0.size

    def step(seed):
        # the forward keeps each sample's radiance for the backward pass
        out = s.render(spp, max_depth=depth, seed=seed, flags=A.ER_RENDER_KEEP_PATHS)
        d = np.zeros_like(out["beauty"])
        d[:, :3] = 2.0 * (out["beauty"][:, :3] - T[:, :3])
        gm, ge, st = s.backward(spp, d, out["samples"], max_depth=depth, seed=seed)
        return out["stats"].ms, st.ms, gm, ge, int(out["stats"].kernel_launches) + int(st.kernel_launches)

    for w in range(max(1, warmup)):
        step(1000 + w)
    clocks = Clocks(0)
    clocks.start()
    time.sleep(0.3)
    t0 = time.perf_counter()
    res = [step(k) for k in range(steps)]
    wall = (time.perf_counter() - t0) / steps
    clk = clocks.stop()
    fwd = float(np.median([r[0] for r in res]))
    bwd = float(np.median([r[1] for r in res]))
    # the replay walk alone (forward render by per-pixel replay, no gradients)
    t0 = time.perf_counter()
    s.render_replay(spp, max_depth=depth, seed=7)
    replay_ms = (time.perf_counter() - t0) * 1e3

    # finite-difference check of the detached estimator (the check of
    # tests/test_gpu_full_configs.py at 256 instead of 4096 spp): central
    # differences of the films' exact FP64 sums on half albedo / roughness
    # and half environment parameters (metallic, drawn from {0, 1}, sits on
    # the estimator's kinks)
    fspp, h = 256, 1e-3
    out = s.render(fspp, max_depth=depth, seed=5)
    d = np.zeros_like(out["beauty"])
    d[:, :3] = 2.0 * (out["beauty"][:, :3] - T[:, :3])
    gm, ge, _ = s.backward(fspp, d, out["samples"], max_depth=depth, seed=5)
    g = np.concatenate([gm.ravel(), ge.ravel()])
    rng = np.random.default_rng(32)
    smooth = np.nonzero(np.arange(m0.size) % 5 != 4)[0]
    half = fd_params // 2
    idx = list(rng.choice(smooth, half, replace=False)) + list(m0.size + rng.choice(e0.size, fd_params - half,
                                                                                        replace=False))

    def loss_exact():
        sums, n = s.read_sums()
        dd = sums / np.maximum(n, 1)[:, None] - T[:, :3].astype(np.float64)
        return float((dd * dd).sum())

    gmax = float(np.abs(g).max())
    errs, skipped = [], 0
    for k in idx:
        vals = []
        for sign in (1, -1):
            m, e = m0.copy(), e0.copy()
            if k < m0.size:
                m.ravel()[k] += sign * h
            else:
                e.ravel()[k - m0.size] += sign * h
            s.render_replay(fspp, max_depth=depth, seed=5, materials=m, env=e, flags=A.ER_RENDER_ACCUM_FP64)
            vals.append(loss_exact())
        fd = (vals[0] - vals[1]) / (2 * h)
        if max(abs(fd), abs(g[k])) < 1e-7 * gmax:
            skipped += 1
            continue
        errs.append(abs(fd - g[k]) / max(abs(fd), abs(g[k])))
    s.close()
    line = {
        "metric": "adjoint full-gradient evaluations/s (512x512, 64 spp forward + 64 spp replay, depth 6)",
        "value": round(1e3 / (fwd + bwd), 4), "unit": "grads/s", "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": round(fwd + bwd, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, reference scene shapes)",
        "config": {"workload": "c4: 64 icospheres (1280 tris each), 1 point light, 256x128 log-normal env; "
                               "L2 loss to a render with other seeded parameters",
                   "parameters": int(n_params), "spp": spp, "max_depth": depth},
        "forward_ms": round(fwd, 2), "backward_ms": round(bwd, 2), "replay_forward_wall_ms": round(replay_ms, 1), "wall_ms_per_step": round(wall * 1e3, 2),
        "backward_msamples_per_s": round(512 * 512 * spp / bwd / 1e3, 2),
        "fd_check": {"params": int(fd_params), "checked": len(errs), "negligible": skipped,
                     "max_rel_err": round(float(max(errs)) if errs else 0.0, 6),
                     "median_rel_err": round(float(np.median(errs)) if errs else 0.0, 6),
                     "h": h, "spp": fspp, "params_from": "albedo, roughness, environment texels",
                     "estimator": "detached sampling (er_render_replay), FP64 film sums"},
        "gpu_launches": int(np.median([r[4] for r in res])),  # per step: forward + backward
    }
    if clk:
        line["clocks"] = clk
    return line


def launch_rays(args):
    """Rays in trace launch b of a 1-spp wave at sample index 1 (the first
    warm-up step of the default run): extension rays of bounce b plus shadow
    rays of bounce b-1, from the ray counters of depth-limited renders."""
    from eleven import _abi as A
    from eleven import _lib
    arrays, max_depth, cfg = make_scene(args.config)
    scene = _lib.Scene(arrays)
    b = args.launch_rays

    def counts(depth):
        if depth == 0:
            return 0, 0
        st = scene.render(spp=1, max_depth=depth, sample_begin=1, flags=A.ER_RENDER_NO_OUTPUT)["stats"]
        return st.rays_closest, st.rays_shadow

    c_b1, _ = counts(b + 1)
    c_b, s_b = counts(b)
    _, s_bm1 = counts(b - 1) if b >= 1 else (0, 0)
    ext = c_b1 - c_b
    shadow = s_b - s_bm1
    print(json.dumps({"launch": b, "extension_rays": int(ext), "shadow_rays": int(shadow),
                      "rays": int(ext + shadow), "config": args.config}))
    return 0


def main():
    args = parse()
    if args.launch_rays >= 0:
        return launch_rays(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "c2":
        return run_batch(args)
    if args.config == "c4":
        return run_adjoint(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
