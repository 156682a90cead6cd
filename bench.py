"""Benchmark: FBP of one 2048 x 2048 slice from 1800 views x 2048 rays
(Ram-Lak filter + slant-stack backprojection), in GUPS = (pixels x views)
updates per second.

Workload (seeded synthetic, no dataset): 40 random ellipses (centres uniform
in the unit disk, semi-axes U(0.02, 0.4), angles U(0, pi), densities
U(0, 1)); transmission sinogram = slant-stack Radon scaled to a maximum
attenuation of 3, Poisson counts at I0 = 1e4 per ray, -log(counts / I0) with
counts >= 1.  One step = one rg_fbp call (filter + backprojection) on a
resident sinogram.  The sinogram (14.7 MB) fits in L2, so L2 is flushed
(160 MiB write, above the 129 MB L2) before every timed step and the step
time is the sum of per-step CUDA-event intervals.

Also reported on the same line:
- the backprojection call alone against its shared-memory roofline (8 B of
  shared memory per interpolated update, one 128-byte wavefront per SM per
  clock), with its measured DRAM traffic against the HBM peak;
- the end-to-end time of the same call with pinned host buffers and both
  copies inside the timed region;
- `osem`: the EM/OSEM half of the metric -- plain EM 100 iterations and OSEM
  10 x 10 on a 1024^2, 720-view emission slice, and the batched uneven OSEM
  (256 slices, 10 subsets x 20 iterations, one persistent batch per
  sub-iteration, graph-captured) against the plain one-slice-per-call form;
- the reference algorithm on the host cores (oracle port, a bounded sample
  of 1/32 of the step spread over the image and the views).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, A, R = 2048, 1800, 2048
METRIC = "FBP GUPS (2048^2 image, 1800 views, 2048 rays; Ram-Lak + slant-stack BP)"
UNIT = "GUPS"
UPDATES = N * N * A
# ncu (dram__bytes_read.sum + dram__bytes_write.sum) of one backprojection
# call at this size (profiles/bp_rot_2048x1800_ncu.md): k_pair_quads reads
# the sinogram (14.9 MB); k_gather_rot_tma reads the quads (29.5 MB, which
# ncu's cache flush between kernels sends to DRAM) and the zeroed image that
# the two partial sums per pixel are added to (16.8 MB).
BP_TRAFFIC_BYTES = 14850304 + 46378496
# kernels of one FBP step: k_to_am, k_filter_fft (which writes the
# backprojection's quads and zeroes the output), k_gather_rot_tma
LAUNCHES_PER_FBP = 3


def smem_roofline(updates, ms, sms, sm_mhz, traffic, compulsory, hbm_peak, hbm_kind):
    """Roofline of the paired backprojection gather.

    Its bound is shared-memory bandwidth, not HBM: every update reads one
    8-byte sample pair (the view's; the partner view's pair arrives in the
    same 128-bit load) from shared memory, and an SM serves one 128-byte
    wavefront per clock, so at most 16 updates per SM per clock.  The
    8 B/update "gather-byte" figure therefore counts shared-memory bytes; a
    staged sample serves ~1000 updates, and DRAM carries only the sinogram,
    the sample quads and the output.  `hbm` reports the measured DRAM
    traffic of the call (ncu) over its CUDA-event time against the HBM peak.
    """
    mhz = sm_mhz or 2070.0
    peak = 128.0 * sms * mhz * 1e6 / 1e9               # GB/s of shared-memory wavefronts
    got = 8.0 * updates / (ms * 1e-3) / 1e9
    dram = traffic / (ms * 1e-3) / 1e9
    return {"bound": "smem", "achieved": round(got, 1), "peak": round(peak, 1), "unit": "GB/s",
            "frac": round(got / peak, 3), "traffic": traffic,
            "algorithmic_bytes": 8 * updates,
            "model": "8 B of shared memory per (pixel, view) update (one sample pair); "
                     "one 128-byte shared-memory wavefront per SM per clock = 16 updates per "
                     "SM per clock",
            "peak_source": f"derived: 128 B x {sms} SMs x {mhz:.0f} MHz (SM clock sampled "
                           f"during the run); MEASURED_PEAKS.json has no shared-memory figure",
            "gups": {"achieved": round(updates / (ms * 1e-3) / 1e9, 1),
                     "peak": round(16.0 * sms * mhz * 1e6 / 1e9, 1)},
            "hbm": {"achieved_gbs": round(dram, 1), "peak": hbm_peak,
                    "peak_source": f"{hbm_kind} (MEASURED_PEAKS.json hbm_gbs)",
                    "frac": round(dram / hbm_peak, 4),
                    "traffic_bytes": traffic, "compulsory_bytes": compulsory,
                    "traffic_over_compulsory": round(traffic / compulsory, 2),
                    "note": "DRAM bytes of one call (ncu dram__bytes_read.sum + "
                            "dram__bytes_write.sum of k_pair_quads + k_gather_rot_tma); "
                            "compulsory = sinogram read + image written once"}}


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------
# Clock sampling during the timed region

class Clocks:
    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None
        self.t = None

    def start(self):
        cmd = ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,"
               "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "50"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append((time.perf_counter(), parts))

    def wait_first(self, timeout=5.0):
        """Block until nvidia-smi has produced its first sample (its start-up
        takes a few hundred ms), so that the sampling covers the timed steps."""
        t0 = time.perf_counter()
        while self.proc and not self.samples and time.perf_counter() - t0 < timeout:
            time.sleep(0.02)

    def stop(self, t_from=None, t_to=None):
        """Median SM clock and the throttle reasons over the samples taken in
        [t_from, t_to] (all samples when no window is given)."""
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.proc = None
        if self.t:
            self.t.join(timeout=2)
            self.t = None
        got = [p for t, p in self.samples
               if (t_from is None or t >= t_from) and (t_to is None or t <= t_to)]
        if not got:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in got if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in got if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in got for k in range(4)
                          if s[3 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(got)}


# ----------------------------------------------------------------------------
# CPU baseline (bounded sample of the same workload on the host cores)

CPU_SAMPLE = 32          # the CPU legs process 1/32 of a step


def cpu_fbp_sample(sino_np):
    """One bounded sample of the FBP step on the host cores: 1/32 of the
    step's work in both of its legs, spread over the whole input.
    - filter: every 32nd view, Ram-Lak by numpy FFT (zero-padded linear
      convolution; pyraft filters by numpy FFT, pyraft/filters/filters.py:13-68);
    - backprojection: every 32nd image row (64 of 2048), the FP64 oracle port
      of raft_backprojection_slantstack (raft/raft_backprojection_slantstack.c:
      121-180) on all host cores.
    Returns (seconds, updates, description, cores, kind); updates = the
    backprojection updates of the sampled rows (pixels x views)."""
    import numpy as np
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    rows = N // CPU_SAMPLE
    dt = 2.0 / (R - 1)
    t0 = time.perf_counter()
    O.ramlak_fft(sino_np[:, ::CPU_SAMPLE], dt)
    s_filter = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.backprojection_rowstep(sino_np, N, CPU_SAMPLE // 2, CPU_SAMPLE, rows, threads=cores)
    s_bp = time.perf_counter() - t0
    sample = (f"1/{CPU_SAMPLE} of the FBP step, spread over the input: Ram-Lak by numpy FFT of "
              f"one view in {CPU_SAMPLE} ({len(range(0, A, CPU_SAMPLE))} of {A}, one thread) and "
              f"the FP64 oracle port of raft_backprojection_slantstack on one image row in "
              f"{CPU_SAMPLE} ({rows} of {N}, {cores} threads); GUPS = the sampled rows' pixel x view "
              f"updates / sample time (filter {1e3 * s_filter:.0f} ms + backprojection "
              f"{1e3 * s_bp:.0f} ms)")
    return s_filter + s_bp, rows * N * A, sample, cores, "port"


def bench_config(world):
    """The `config` object of both arms (identical, so the two lines compare)."""
    return {"workload": "FBP 2048x2048, 1800 views in [0,pi), 2048 rays, Ram-Lak + "
                        "slant-stack backprojection, one slice per GPU",
            "image": N, "views": A, "rays": R, "filter": "ramlak",
            "l2": "flushed (160 MiB write) before every timed step; step time = sum "
                  "of per-step CUDA-event intervals",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


# ----------------------------------------------------------------------------

def make_sinogram(torch, rg, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    desc = rg.random_ellipses(40, rng)
    ph = rg.phantom_fromdesc((N, N), desc, device=True)
    # slant-stack rows are bottom-up: flip the top-down raster
    ph = rg.gpu_image(torch.flip(ph.data, dims=[0]).contiguous())
    p = rg.radon(ph, (R, A), rg.radon_method.SLANTSTACK)
    mu = 3.0 / float(p.data.max())
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    counts = torch.poisson(1e4 * torch.exp(-p.data * mu), generator=gen).clamp_(min=1.0)
    s = -torch.log(counts / 1e4)
    return s.contiguous()


def osem_batch_sizes(nslices, seed):
    """(N, views) of every slice of the config-5 batch: N uniform over
    {256, 512, 1024, 2048}, views uniform in [180, 1800], rays = N."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [(int(rng.choice([256, 512, 1024, 2048])), int(rng.integers(180, 1801)))
            for _ in range(nslices)]


def make_osem_batch(torch, rg, idx, sizes, seed):
    """Sinograms of slices `idx` of the config-5 batch: random-ellipse
    emission phantoms, Poisson counts with mean 50 per bin.  Each slice draws
    from its own seeded generators, so a slice is the same whichever rank
    builds it.  Returns (rays, views) GPU tensors."""
    import numpy as np
    sinos = []
    for i in idx:
        n, a = sizes[i]
        rng = np.random.default_rng([seed, i])
        desc = rg.random_ellipses(12, rng)
        ph = rg.phantom_fromdesc((n, n), desc, device=True)
        ph = rg.gpu_image(torch.flip(ph.data, dims=[0]).abs().contiguous())
        p = rg.radon(ph, (n, a), rg.radon_method.SLANTSTACK).data
        lam = p.clamp(min=0) * (50.0 / max(float(p.mean()), 1e-9))
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed * 1000003 + i)
        sinos.append(torch.poisson(lam, generator=gen).contiguous())
    return sinos


def osem_compare(torch, rg, nslices, niter, nsubsets, plain_stride, seed=7, rank=0, world=1,
                 runs=3):
    """Batched graph-captured OSEM vs the plain one-slice-per-call form on
    the same slices.  With several ranks (one per GPU) the slices are
    partitioned by cost (pyraft_gb300.shard) and the batched time is the max
    over ranks (median of `runs` full runs).  The plain form runs on rank 0
    only, on every `plain_stride`-th of its slices (all of them for stride
    1), and its time is scaled to the whole batch by the sampled slices'
    share of sum(N^2 x views)."""
    import numpy as np
    from pyraft_gb300 import _native, shard
    from pyraft_gb300.raftypes import rg_image
    L = _native.load()
    sizes_all = osem_batch_sizes(nslices, seed)
    mine = shard.rank_slices([n * n * a for n, a in sizes_all], rank, world)
    sizes = [sizes_all[i] for i in mine]
    sinos = make_osem_batch(torch, rg, mine, sizes_all, seed)
    ns = len(mine)
    S = (_native.RG_IMAGE * ns)(*[rg_image(rg.gpu_image(s, (0.0, 1.0), (math.pi, -1.0)))
                                  for s in sinos])
    xs = [torch.ones((n, n), dtype=torch.float32, device="cuda") for n, _ in sizes]
    I = (_native.RG_IMAGE * ns)(*[rg_image(rg.gpu_image(x)) for x in xs])
    wsb = L.rg_osem_batch_workspace(S, I, ns, nsubsets)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream

    def run_batch(it):
        for x in xs:
            x.fill_(1.0)
        _native.check(L.rg_osem_batch(S, I, ns, it, nsubsets, 1, ws.data_ptr(), wsb, sp))
    run_batch(1)                                     # warm-up (plans, graph path)
    torch.cuda.synchronize()
    times = []
    for _ in range(runs):
        if world > 1:
            torch.distributed.barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        run_batch(niter)
        b.record()
        b.synchronize()
        times.append(shard.max_over_ranks(a.elapsed_time(b) * 1e-3, device="cuda"))
    t_batch = statistics.median(times)
    upd = sum(2.0 * n * n * v for n, v in sizes_all) * niter
    res = {
        "slices": nslices, "iterations": niter, "subsets": nsubsets, "n_gpus": world,
        "batched_slices_per_s": round(nslices / t_batch, 3),
        "batched_s": round(t_batch, 3),
        "batched_runs": runs,
        "batched_gups": round(upd / t_batch / 1e9, 1),
    }
    if rank != 0:
        return res
    pick = list(range(0, ns, max(1, plain_stride)))
    host = {k: sinos[k].cpu().numpy() for k in pick}
    out = np.zeros((2048, 2048), dtype=np.float32)
    t0 = time.perf_counter()
    for k in pick:
        n, v = sizes[k]
        _native.check(L.rg_em_plain_host(out.ctypes.data, host[k].ctypes.data, n, n, v, niter,
                                         nsubsets))
    t_plain = time.perf_counter() - t0
    frac = sum(sizes[k][0] ** 2 * sizes[k][1] for k in pick) / \
        sum(n * n * v for n, v in sizes_all)
    t_plain_all = t_plain / frac
    res.update({
        "plain_slices_per_s": round(nslices / t_plain_all, 3),
        "plain_s": round(t_plain_all, 3),
        "plain_timed_slices": len(pick),
        "plain_timed_s": round(t_plain, 3),
        "plain_note": (f"one GPU, every {max(1, plain_stride)}th slice of rank 0 timed "
                       f"({len(pick)} slices, {100 * frac:.1f} % of the batch's N^2 x views), "
                       f"scaled by that share"),
        "speedup_per_gpu": round(t_plain_all / t_batch / world, 2),
    })
    return res


def em_run(torch, rg, n=1024, nviews=720, seed=5, only=None, osem_iters=10):
    """Config-3 workload: 1024^2 emission slice (random ellipses), 720 views,
    1024 rays, Poisson counts with mean 50 per bin; plain EM 100 iterations
    vs OSEM 10 interleaved subsets x 10 iterations, x0 = 1, FP64
    sensitivities.  One slice per call through rg_em.  only="em" or "osem"
    runs one of the two (profiling); osem_iters sets the OSEM iterations."""
    import numpy as np
    from pyraft_gb300 import _native
    from pyraft_gb300.raftypes import rg_image
    L = _native.load()
    rng = np.random.default_rng(seed)
    ph = rg.phantom_fromdesc((n, n), rg.random_ellipses(40, rng), device=True)
    ph = rg.gpu_image(torch.flip(ph.data, dims=[0]).abs().contiguous())
    p = rg.radon(ph, (n, nviews), rg.radon_method.SLANTSTACK).data
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    y = torch.poisson(p.clamp(min=0) * (50.0 / float(p.mean())), generator=gen).contiguous()
    x = torch.ones((n, n), device="cuda")
    S = rg_image(rg.gpu_image(y, (0.0, 1.0), (math.pi, -1.0)))
    X = rg_image(rg.gpu_image(x))
    sp = torch.cuda.current_stream().cuda_stream
    out = {}
    runs = [("em_100", 100, 1), (f"osem_10x{osem_iters}", osem_iters, 10)]
    for name, it, subsets in [r for r in runs if only is None or r[0].startswith(only)]:
        wsb = L.rg_em_workspace(S, X, _native.RG_SLANTSTACK, subsets)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        x.fill_(1.0)
        _native.check(L.rg_em(S, X, _native.RG_SLANTSTACK, 1, subsets, ws.data_ptr(), wsb, sp))
        ts = []
        for _ in range(3):                           # median of three full runs
            x.fill_(1.0)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            _native.check(L.rg_em(S, X, _native.RG_SLANTSTACK, it, subsets, ws.data_ptr(), wsb,
                                  sp))
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b) * 1e-3)
        t = statistics.median(ts)
        upd = 2.0 * n * n * nviews * it
        out[name] = {"seconds": round(t, 4), "slices_per_s": round(1.0 / t, 3),
                     "gups": round(upd / t / 1e9, 1)}
    return {"size": n, "views": nviews, **out}


def tvls_run(torch, rg, nslices=64, n=512, nviews=360, steps=200, seed=11):
    """Config-4 workload: 64 random-ellipse slices of 512^2, 360 views, 512
    rays, Gaussian noise sigma = 1% of max; TV-regularised least squares
    (lambda 1e-3) with 200 Adam steps through the autograd Radon pair."""
    import numpy as np
    from pyraft_gb300 import autograd as AG, recon
    rng = np.random.default_rng(seed)
    xs = []
    for _ in range(nslices):
        ph = rg.phantom_fromdesc((n, n), rg.random_ellipses(40, rng), device=True)
        xs.append(torch.flip(ph.data, dims=[0]))
    x_true = torch.stack(xs).contiguous()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    y = AG.radon_forward(x_true, n, nviews)
    y = y + 0.01 * float(y.max()) * torch.randn(y.shape, device="cuda", generator=gen)
    recon.tv_ls(y, n, niter=3)                                   # warm-up / plans
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    x, losses = recon.tv_ls(y, n, niter=steps, lam=1e-3, lr=2e-2)
    b.record()
    b.synchronize()
    t = a.elapsed_time(b) * 1e-3
    upd = 2.0 * nslices * n * n * nviews * steps                  # forward + adjoint per step
    err = float(torch.linalg.norm(x - x_true) / torch.linalg.norm(x_true))
    return {"slices": nslices, "size": n, "views": nviews, "steps": steps,
            "seconds": round(t, 3), "ms_per_step": round(1e3 * t / steps, 3),
            "operator_gups": round(upd / t / 1e9, 1), "final_loss": losses[-1],
            "loss_ratio": losses[-1] / losses[0], "rel_error_vs_truth": round(err, 4)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fbp", choices=["fbp", "osem", "tvls", "em"],
                    help="fbp: the headline FBP line; osem: batched uneven OSEM "
                         "(256 slices, 10 subsets x 20 iterations) vs the plain form")
    ap.add_argument("--slices", type=int, default=256)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--plain-stride", type=int, default=4,
                    help="the plain per-call form times every k-th slice of the batch")
    ap.add_argument("--batch-runs", type=int, default=2,
                    help="timed runs of the whole batched OSEM (median)")
    ap.add_argument("--no-osem", action="store_true",
                    help="FBP line without its osem object (quick runs)")
    ap.add_argument("--em-only", choices=["em", "osem"], default=None,
                    help="--workload em: run only EM-100 or only the OSEM part (profiling)")
    ap.add_argument("--osem-iters", type=int, default=10,
                    help="--workload em: OSEM iterations (10 subsets each)")
    args = ap.parse_args()
    rank, world, local = env_rank()
    warm = max(3, args.warmup)

    if args.impl == "reference":
        return reference_arm(args, rank, world, warm)
    if args.workload == "em":
        import torch
        import pyraft_gb300 as rg
        torch.cuda.set_device(local)
        print(json.dumps({"workload": "EM 100 iterations vs OSEM 10x10, 1024^2, 720 views",
                          **em_run(torch, rg, only=args.em_only,
                                   osem_iters=args.osem_iters)}))
        return
    if args.workload == "tvls":
        import torch
        import pyraft_gb300 as rg
        torch.cuda.set_device(local)
        print(json.dumps({"workload": "TV-regularised LS, 64 x 512^2, 360 views, 200 Adam steps",
                          **tvls_run(torch, rg)}))
        return
    if args.workload == "osem":
        import torch
        import pyraft_gb300 as rg
        torch.cuda.set_device(local)
        if world > 1:
            torch.distributed.init_process_group("nccl")
        res = osem_compare(torch, rg, args.slices, args.iters, 10, args.plain_stride,
                           rank=rank, world=world, runs=args.batch_runs)
        if rank == 0:
            print(json.dumps({"workload": "batched uneven OSEM vs plain per-call form",
                              "scaling": "strong (slices partitioned over GPUs by cost)",
                              **res}))
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    import numpy as np
    import torch
    import pyraft_gb300 as rg
    from pyraft_gb300 import _native
    from pyraft_gb300.raftypes import rg_image

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = _native.load()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    sino = make_sinogram(torch, rg, 1234 + rank)                  # (R, A) rays x views
    img = torch.zeros((N, N), dtype=torch.float32, device="cuda")
    S = rg_image(rg.gpu_image(sino, (0.0, 1.0), (math.pi, -1.0)))
    I = rg_image(rg.gpu_image(img))
    ws_bytes = L.rg_fbp_workspace(S, I, _native.RG_FILTER_RAMLAK)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    flush = torch.empty(160 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2

    def step():
        _native.check(L.rg_fbp(S, I, _native.RG_FILTER_RAMLAK, ws.data_ptr(), ws_bytes, sp))

    clocks = Clocks(local)
    clocks.start()
    for _ in range(warm):
        step()
    torch.cuda.synchronize()
    clocks.wait_first()

    # ---- device-resident steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall1 = time.perf_counter()
    wall = wall1 - wall0
    if dist:
        dist.barrier()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
    value = world * UPDATES / (ms * 1e-3) / 1e9

    # ---- backprojection kernel alone (roofline of the dominant kernel)
    filt_am = torch.empty((A, R), dtype=torch.float32, device="cuda")
    FA = rg_image(rg.gpu_image(filt_am.t(), (0.0, 1.0), (math.pi, -1.0)))   # view-major view
    FS = rg_image(rg.gpu_image(sino, (0.0, 1.0), (math.pi, -1.0)))
    fws = L.rg_filter_workspace(FS, _native.RG_FILTER_RAMLAK)
    fwsb = torch.empty(fws, dtype=torch.uint8, device="cuda")
    _native.check(L.rg_filter(FS, FA, _native.RG_FILTER_RAMLAK, fwsb.data_ptr(), fws, sp))
    # a view-major sinogram needs no layout copy, only the paired gathers' quads
    bws = L.rg_backprojection_slantstack_workspace(FA, I)
    bwsb = torch.empty(bws, dtype=torch.uint8, device="cuda")
    bp_ms = []
    for k in range(warm + args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        _native.check(L.rg_backprojection_slantstack(FA, I, bwsb.data_ptr(), bws, sp))
        b.record(stream)
        b.synchronize()
        if k >= warm:
            bp_ms.append(a.elapsed_time(b))
    bp_ms = statistics.mean(bp_ms)
    compulsory = N * N * 4 + R * A * 4
    peak, peak_kind = measured_peaks()
    sms = torch.cuda.get_device_properties(0).multi_processor_count

    # ---- the other operators of the path at the same size (one call each)
    def timed(fn, reps=5):
        out = []
        for k in range(warm + reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            if k >= warm:
                out.append(a.elapsed_time(b))
        return statistics.mean(out)
    src = torch.flip(img, dims=[0]).contiguous()
    sino_out = torch.empty((A, R), dtype=torch.float32, device="cuda")
    SO = rg_image(rg.gpu_image(sino_out.t(), (0.0, 1.0), (math.pi, -1.0)))
    RI = rg_image(rg.gpu_image(src))
    rws = L.rg_radon_slantstack_workspace(RI, SO)
    rwsb = torch.empty(rws, dtype=torch.uint8, device="cuda")
    radon_ms = timed(lambda: _native.check(L.rg_radon_slantstack(RI, SO, rwsb.data_ptr(), rws,
                                                                 sp)))
    aws = L.rg_radon_transpose_slantstack_workspace(FA, I)
    awsb = torch.empty(aws, dtype=torch.uint8, device="cuda")
    adj_ms = timed(lambda: _native.check(L.rg_radon_transpose_slantstack(FA, I, awsb.data_ptr(),
                                                                         aws, sp)))

    # ---- end to end: pinned host sinogram in, image out, through rg_fbp
    h_in = torch.empty((R, A), dtype=torch.float32).pin_memory()
    h_in.copy_(sino.cpu())
    h_out = torch.empty((N, N), dtype=torch.float32).pin_memory()
    d_in = torch.empty_like(sino)
    d_out = torch.empty_like(img)
    S2 = rg_image(rg.gpu_image(d_in, (0.0, 1.0), (math.pi, -1.0)))
    I2 = rg_image(rg.gpu_image(d_out))

    def e2e_step():
        d_in.copy_(h_in, non_blocking=True)
        _native.check(L.rg_fbp(S2, I2, _native.RG_FILTER_RAMLAK, ws.data_ptr(), ws_bytes, sp))
        h_out.copy_(d_out, non_blocking=True)

    for _ in range(warm):
        e2e_step()
    torch.cuda.synchronize()
    e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        e2e_step()
        b.record(stream)
        b.synchronize()
        e_ms.append(a.elapsed_time(b))
    e_ms = statistics.mean(e_ms)
    if dist:
        t = torch.tensor([e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e_ms = float(t)
    ok = bool(torch.isfinite(h_out).all())

    # ---- end to end, streamed: the same calls for a stream of slices.  Two
    # device buffer sets; step k's upload, FBP and download run on three
    # streams, so the upload of step k+1 and the download of step k-1
    # overlap the FBP of step k.  Every step still uploads its sinogram from
    # pinned host memory, flushes L2 and downloads its image inside the timed
    # region; the time is the whole run's, first upload to last download.
    s_in, s_cp, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    d_ins = [torch.empty_like(sino) for _ in range(2)]
    d_outs = [torch.empty_like(img) for _ in range(2)]
    h_outs = [torch.empty((N, N), dtype=torch.float32).pin_memory() for _ in range(2)]
    S_p = [rg_image(rg.gpu_image(t, (0.0, 1.0), (math.pi, -1.0))) for t in d_ins]
    I_p = [rg_image(rg.gpu_image(t)) for t in d_outs]
    torch.cuda.synchronize()

    def run_stream(K):
        up = [torch.cuda.Event() for _ in range(K)]
        done = [torch.cuda.Event() for _ in range(K)]
        down = [torch.cuda.Event() for _ in range(K)]
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(s_in)
        for k in range(K):
            b = k % 2
            if k >= 2:
                s_in.wait_event(done[k - 2])       # d_ins[b] read by step k-2's FBP
            with torch.cuda.stream(s_in):
                d_ins[b].copy_(h_in, non_blocking=True)
            up[k].record(s_in)
            s_cp.wait_event(up[k])
            if k >= 2:
                s_cp.wait_event(down[k - 2])       # d_outs[b] downloaded by step k-2
            with torch.cuda.stream(s_cp):
                flush.zero_()
            _native.check(L.rg_fbp(S_p[b], I_p[b], _native.RG_FILTER_RAMLAK, ws.data_ptr(),
                                   ws_bytes, s_cp.cuda_stream))
            done[k].record(s_cp)
            s_out.wait_event(done[k])
            with torch.cuda.stream(s_out):
                h_outs[b].copy_(d_outs[b], non_blocking=True)
            down[k].record(s_out)
        t1.record(s_out)
        t1.synchronize()
        return t0.elapsed_time(t1) / K

    run_stream(warm)
    # three runs of `steps` slices each, the median reported: one run's
    # throughput follows the host thread that enqueues it, and a stall of
    # that thread (seen once in tens of runs) starves the streams
    p_runs = [run_stream(args.steps) for _ in range(3)]
    p_ms = statistics.median(p_runs)
    if dist:
        t = torch.tensor([p_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        p_ms = float(t)
    ok = ok and bool(torch.isfinite(h_outs[0]).all()) and bool(torch.isfinite(h_outs[1]).all())
    ok = ok and bool(torch.allclose(h_outs[0], h_out)) and bool(torch.allclose(h_outs[1], h_out))
    wall_end = time.perf_counter()
    # nvidia-smi samples every 50 ms: a short timed region may hold none, in
    # which case the window widens to every GPU phase after it (the same
    # kernels under the same load: kernel-only and end-to-end steps).
    clk = clocks.stop(wall0, wall1)
    clk["window"] = "timed steps"
    if clk["sm_mhz"] is None:
        clk = clocks.stop(wall0, wall_end)
        clk["window"] = "timed steps + kernel-only + end-to-end steps"

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": warm, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded random-ellipse transmission sinogram, Poisson I0=1e4)",
        "config": bench_config(world),
        "e2e": {"value": round(world * UPDATES / (p_ms * 1e-3) / 1e9, 3), "unit": UNIT,
                "h2d_bytes_per_step": R * A * 4, "d2h_bytes_per_step": N * N * 4,
                "ms_per_step": round(p_ms, 4), "api": "rg_fbp (C ABI), pinned host buffers",
                "mode": "streamed slices: step k+1's upload and step k-1's download overlap "
                        "step k's FBP (two buffer sets, three CUDA streams); L2 flushed before "
                        "every FBP inside the timed region; time = first upload to last "
                        "download over all steps; the median of three such runs",
                "runs_ms_per_step": [round(x, 4) for x in p_runs],
                "serial": {"value": round(world * UPDATES / (e_ms * 1e-3) / 1e9, 3),
                           "ms_per_step": round(e_ms, 4),
                           "mode": "upload, FBP, download back to back on one stream, "
                                   "per-step CUDA events"},
                "finite_and_equal": ok},
        "roofline": {"kernel": "k_gather_rot_tma<0> (backprojection, views paired a quarter "
                               "turn apart, windows staged by TMA; timed as the call, with its "
                               "k_pair_quads prepass, which also zeroes the output)",
                     "kernel_ms": round(bp_ms, 4),
                     **smem_roofline(UPDATES, bp_ms, sms, clk["sm_mhz"], BP_TRAFFIC_BYTES,
                                     compulsory, peak, peak_kind)},
        "ops": {"radon_gups": round(R * A * N / (radon_ms * 1e-3) / 1e9, 1),
                "radon_ms": round(radon_ms, 4),
                "adjoint_gups": round(UPDATES / (adj_ms * 1e-3) / 1e9, 1),
                "adjoint_ms": round(adj_ms, 4),
                "backprojection_gups": round(UPDATES / (bp_ms * 1e-3) / 1e9, 1),
                "note": "single calls at 2048^2 x 1800 (view-major sinogram), L2 flushed"},
        "gpu_launches": LAUNCHES_PER_FBP * args.steps,
        "clocks": clk,
        "wall_s_timed_region": round(wall, 3),
    }
    if not args.no_osem:
        # The metric's EM/OSEM half, after the FBP measurements (it does not
        # touch their timed region).
        em = em_run(torch, rg)
        batch = osem_compare(torch, rg, args.slices, args.iters, 10, args.plain_stride,
                             rank=rank, world=world, runs=args.batch_runs)
        line["osem"] = {
            "unit": "slices/s",
            "em_slice": {"workload": "EM 100 iterations and OSEM 10 subsets x 10 iterations, "
                                     "1024^2 emission slice, 720 views, 1024 rays, Poisson "
                                     "counts (mean 50 per bin), x0 = 1, one rg_em call each",
                         **em},
            "batch": {"workload": "batched uneven OSEM: 256 slices, N in {256,512,1024,2048}, "
                                  "views in [180,1800], rays = N, 10 subsets x 20 iterations; "
                                  "batched = rg_osem_batch (persistent grids, graph-captured "
                                  "sub-iterations, resident sinograms); plain = rg_em_plain_host "
                                  "per slice (host buffers, five launches per sub-iteration)",
                      **batch},
        }
    if rank == 0:
        t_cpu, upd_cpu, sample, cores, kind = cpu_fbp_sample(h_in.numpy().astype(np.float64))
        line["cpu_baseline"] = {"value": round(upd_cpu / t_cpu / 1e9, 4), "unit": UNIT,
                                "cores": cores, "kind": kind, "sample": sample,
                                "sample_ms": round(1e3 * t_cpu, 1)}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def reference_arm(args, rank, world, warm):
    """The reference's CPU algorithm on the host cores (the oracle port; the
    compiled reference does not travel to the GPU machine), same metric and
    config as the GPU arm.  Each step is one bounded sample: 1/32 of the FBP
    step spread over the input (cpu_fbp_sample), and the value is the
    sample's updates over its measured time, so steps x ms_per_step is the
    arm's real timed region.  Under torchrun only rank 0 works."""
    if rank != 0:
        return
    import numpy as np
    rng = np.random.default_rng(1234)
    sino = rng.random((R, A))
    steps, upd = [], 0
    for k in range(warm + args.steps):
        t, upd, sample, cores, kind = cpu_fbp_sample(sino)
        if k >= warm:
            steps.append(t)
    t = statistics.mean(steps)
    v = upd / t / 1e9
    print(json.dumps({
        "metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": warm, "ms_per_step": round(t * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (uniform random sinogram of the FBP shape)", "impl": "reference",
        "config": bench_config(world),
        "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": sample},
        "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


if __name__ == "__main__":
    main()
