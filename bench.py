"""Benchmark: GALMOD + beam + log L evaluations per second on the 160x160x128 GLOBAL workload.

One step = one batch of likelihood evaluations of the GLOBAL 3DFIT problem (40 rings, VROT VDISP INC PA free
per ring: the base parameters and one step of each of the 160 free parameters, 161 evaluations), each a full
Monte-Carlo GALMOD model in its box, its beam convolution (30"x20" beam, 13x9 kernel) and the masked residual
reduced to log L. Synthetic mock data (no public dataset): the model of the rings plus beam-correlated noise
(sigma 0.5% of the peak), likelihood voxels the 3-sigma mask of the noise-free model dilated by one beam and
+-3 channels.

  value  device throughput with the batch resident in HBM (bbgpu_eval_run), evaluations / s;
  e2e    the same through the C ABI from host arrays: ring values -> sub-ring tables (host) -> upload ->
         device -> download of the sums -> log L, evaluations / s.

python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl reference]
Under torchrun (N > 1) each rank evaluates its own batch on its GPU (replicas: the evaluations are independent),
the time is the max over ranks and value the evaluations of all ranks / that time.
"""

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GALMOD+beam+logL evals/s (160x160x128 f32)"
UNIT = "evals/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None
        self.path = os.path.join("/tmp", f"bb_clocks_{os.getpid()}.csv")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(batch):
    """The device model, likelihood and one batch of ring-value rows (base + one step per free parameter)."""
    from bbarolo2_gb300 import configs, engine
    from scipy import ndimage
    cube, rings = configs.global160(galmodtype="MC")
    dm = engine.DiskModel(cube)
    truth = dm.array(rings, seed=1)
    rms = 0.005 * float(truth.max())
    g = np.random.default_rng(1)
    noise = dm.convolve_planes(g.normal(0., rms, truth.shape))
    noise *= rms / np.std(noise)
    data = (truth + noise).astype(np.float32)
    h = cube.Head()
    rad = abs(h.Bmaj() / h.Cdelt(1))
    yy, xx = np.mgrid[-int(rad) - 1:int(rad) + 2, -int(rad) - 1:int(rad) + 2]
    disk = (xx * xx + yy * yy) <= rad * rad
    mask = ndimage.binary_dilation(truth > 3 * rms, structure=disk[None])
    mask = ndimage.binary_dilation(mask, structure=np.ones((7, 1, 1), bool))
    L = engine.BatchLikelihood(dm, data, mask, maskmode=2, sigma=rms)
    # DENS is not fitted and the geometry is free: the deconvolved profile is recomputed at every evaluation
    # (bbarolo/bayesian/likelihood.py:595-596), with the noise correlated over the beam
    bmaj, bmin = abs(h.Bmaj()), abs(h.Bmin())
    beam_area = math.pi * bmaj * bmin / (4. * math.log(2.)) / abs(h.Cdelt(0) * h.Cdelt(1))
    mom0, mrms, ok = L.data_maps()
    L.set_profile(rings, mom0, mrms, ok, smooth=0.3, corr=beam_area, beam_arcsec=bmaj * 3600.)
    return dm, L, rings, step_rows(rings, batch), data, mask


RING_KEYS = ("radii", "xpos", "ypos", "vsys", "vrot", "vdisp", "vrad", "vvert", "dvdz", "zcyl", "dens", "z0", "inc",
             "phi", "z0thick", "fthick", "vdispthick")


def ring_rows(rings):
    """The ring values (17, nr) of a ring set, in the order of RING_KEYS."""
    return np.vstack([np.asarray(getattr(rings, k), float) for k in RING_KEYS])


def step_rows(rings, batch):
    """The ring values of a gradient batch: the base point, then one step of VROT, VDISP, INC or PA of one ring
    per member: forward steps (GLOBAL's Jacobian columns, 1 + 160 points), then backward steps (a
    central-difference gradient, 2n + 1 = 321 points)."""
    base = ring_rows(rings)
    rows = np.repeat(base[None], batch, axis=0)
    free = [(4, 2.0), (5, 0.5), (12, 0.5), (13, 0.5)]       # vrot, vdisp, inc, phi steps
    k = 1
    for sign in (1.0, -1.0):
        for j in range(rings.nr):
            for row, step in free:
                if k < batch:
                    rows[k, row, j] += sign * step
                    k += 1
    return rows


# ncu summaries (profiles/) with the DRAM traffic of a kernel's launch at the default batch
# (the convolution by variant: the float32 kernel and the tensor-core tf32x3 kernel are different launches)
TRAFFIC = {"mc_deposit": "k_mc_deposit_px.global160_b161.dram.txt", "mc_replay": "mc_replay.global160_b161.dram.txt",
           "conv_resid/f32": "k_conv_resid.global160_b161.dram.txt",
           "conv_resid/tf32x3": "k_conv_tc.global160_b161.dram.txt"}


def measured_traffic(kernel, batch, members=None):
    """DRAM bytes (read + write) of one launch of the kernel at this batch (and number of members in the
    launch), from its committed ncu summary, or None (not captured at this batch)."""
    name = TRAFFIC.get(kernel)
    if not name:
        return None
    try:
        vals = {}
        with open(os.path.join(ROOT, "profiles", name)) as f:
            for line in f:
                if "=" in line and not line.startswith(" "):
                    k, v = line.split("=", 1)
                    vals[k.strip()] = v.strip()
        if int(vals["batch"]) != batch or (members is not None and int(vals.get("members", -1)) != members):
            return None
        return int(vals["traffic_bytes_per_launch"])
    except (OSError, KeyError, ValueError):
        return None


def max_over_ranks(t, dist):
    """The largest of the ranks' times (replicas: the job ends with the slowest rank); t on one rank without
    torch.distributed. NCCL reduces a CUDA tensor, gloo a CPU one."""
    if not dist:
        return t
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    x = torch.tensor([float(t)], dtype=torch.float64, device=dev)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def throughput(units_per_rank, steps, world, t):
    """Whole-job throughput of N replicas: the units of all ranks / the max-over-ranks time."""
    return units_per_rank * steps * world / t


def algorithmic(dm, L, sr, nv, descs, mc_members=None):
    """Algorithmic bytes / flops per launch of the kernels (summed over the batch; the first MC deposit launch
    covers mc_members of them, the members that deposit all their clouds)."""
    st = dm.setup
    nz = st.nsubs
    ky, kx = dm.cfield.shape
    taps = int(np.count_nonzero(dm.cfield))
    vox = sum((int(d["bhi0"]) - int(d["blo0"])) * (int(d["bhi1"]) - int(d["blo1"])) * nz for d in descs)
    # MC deposit: the clouds (16 B) and their velocity deviates (4 B each) are one table shared by the batch,
    # read once; each member's model is written once (4 B per voxel)
    from bbarolo2_gb300.galmod import cloud_counts
    ncl, nsubcl = cloud_counts(st, sr[0], nv[0])
    B = len(descs)
    mc_bytes = 4 * nsubcl + 16 * ncl + 4 * vox * (B if mc_members is None else mc_members) // B
    conv_flops = 2.0 * taps * vox
    conv_bytes = 4 * vox * 2 + vox // 1        # model read + data read (+ mask folded in the data)
    return dict(mc_deposit=("hbm", mc_bytes), conv_resid=("fp32", conv_flops), conv_bytes=conv_bytes,
                deposits=B * nsubcl, voxels=vox, taps=taps, kernel=[ky, kx],
                # per launch, for m members: the deposit reads the deviate table once and 16 B per cloud and
                # member, and writes the models; the replay reads member 0's records of its channel counts
                # (136 B a cloud) once and writes the models; the convolution reads the models and the data
                # once (the data of the box is the same for all members)
                mc_deposit_bytes=lambda m: 4 * nsubcl + 16 * ncl * m + 4 * vox * m // B,
                mc_replay_bytes=lambda m: 136 * ncl + 4 * vox * m // B,
                conv_resid_bytes=lambda m: 4 * vox * m // B + 4 * vox // B)


def cpu_leg(dm, L, rows, rings, data, mask, cores=None, sample=None, steps=1):
    """The reference algorithm on the host cores (oracle C kernels + scipy FFT), bounded sample."""
    from oracle import cpu_baseline
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    payload = cpu_baseline.setup_payload(dm, sr, nv, boxes, 1, data, L.mask, L.maskmode, like=L, rows=rows,
                                         proto=rings)
    pool = cpu_baseline.Pool(payload, cores)
    n = sample or min(len(rows), 2 * pool.cores)
    pool.run(range(min(pool.cores, len(rows))))              # warm-up (FFT plans, caches)
    vals = []
    for _ in range(steps):
        _, wall = pool.run(range(n))
        vals.append(n / wall)
    pool.close()
    return vals, pool.cores, n


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=161)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-analytic", action="store_true", help="skip the ANALYTIC GALMOD leg")
    ap.add_argument("--no-central", action="store_true", help="skip the 321-point central-difference batch")
    ap.add_argument("--no-bayes", action="store_true",
                    help="skip the 256x256x192 batch of 1024 points and the BAYESIAN fit")
    ap.add_argument("--bayes-nb", type=int, default=1024,
                    help="points per launch of the 256x256x192 batch (the BAYESIAN workload: 1024)")
    ap.add_argument("--no-bayes-fit", action="store_true", help="skip the BAYESIAN fit time (plain and screened)")
    ap.add_argument("--no-classic", action="store_true", help="skip the CLASSIC fit of the 64x64x64 workload")
    ap.add_argument("--no-ragged", action="store_true", help="skip the heterogeneous batch of 128 galaxies")
    ap.add_argument("--no-wind", action="store_true", help="skip the WINDFIT normal equations (Circinus shapes)")
    ap.add_argument("--no-galwind", action="store_true", help="skip the GALWIND WTYPE 1 model")
    ap.add_argument("--wind-only", action="store_true",
                    help="run the WINDFIT and GALWIND legs alone and print their line (for profiling them)")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the per-variant convolution times and errors")
    ap.add_argument("--no-random", action="store_true",
                    help="skip the batch of independent points and the gradient batch without shared ring maps")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.wind_only:
        out = {"wind": wind_leg(args, dist, world, cpu=rank == 0 and not args.no_cpu)}
        if not args.no_galwind:
            out["galwind"] = galwind_leg(args, dist, world, cpu=rank == 0 and not args.no_cpu)
        if rank == 0:
            print(json.dumps(out))
        return 0
    if args.impl == "reference":
        if rank != 0:
            return 0
        return reference_arm(args, world)
    from bbarolo2_gb300 import _lib, build
    build.build()
    dm, L, rings, rows, data, mask = workload(args.batch)
    ctx = dm.ctx
    B = rows.shape[0]
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    # ---- device-resident throughput
    ctx.check(ctx.L.bbgpu_eval_upload(ctx.h, _lib.MC, B, sr.shape[2], _lib.ptr(sr), _lib.ptr(nv), _lib.ptr(descs)))
    ms = L._maps_sr
    ctx.check(ctx.L.bbgpu_eval_upload_profile(ctx.h, ms.shape[2], _lib.ptr(ms), _lib.ptr(L._prof["widx"]),
                                              _lib.ptr(L._prof["wval"])))
    for _ in range(args.warmup):
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
    ctx.check(ctx.L.bbgpu_sync(ctx.h))
    clk = Clocks(local)
    if dist:
        dist.barrier()
    l0 = ctx.launches
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
    ctx.check(ctx.L.bbgpu_sync(ctx.h))
    dt = time.perf_counter() - t0
    launches = ctx.launches - l0
    graph_replays, graph_kernels = ctx.graph_stats()
    dt = max_over_ranks(dt, dist)
    if dist:
        dist.barrier()
    ss = np.zeros(B)
    lg = np.zeros(B)
    ctx.check(ctx.L.bbgpu_eval_download(ctx.h, _lib.ptr(ss), _lib.ptr(lg)))
    value = throughput(B, args.steps, world, dt)
    # ---- per-kernel device times (CUDA events on the context's stream)
    ctx.set_option(_lib.OPT_TIMING, 1)
    ktimes = {}
    for _ in range(3):
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
        for kname, v in ctx.run_times().items():
            ktimes.setdefault(kname, []).append(v)
    ctx.set_option(_lib.OPT_TIMING, 0)
    kt = {k: float(np.median(v)) for k, v in ktimes.items()}
    # ---- end to end through the C ABI from host arrays
    for _ in range(max(1, args.warmup // 2)):
        L.evaluate(rows, rings, seed=1)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = L.evaluate(rows, rings, seed=1)
    te = time.perf_counter() - t0
    te = max_over_ranks(te, dist)
    h2d, d2h = ctx.transfer_bytes()
    clocks = clk.stop()
    e2e = throughput(B, args.steps, world, te)
    # ---- roofline of the dominant kernel
    hbm, bf16, src = peaks()
    # (the last run of the batch above: how many members were computed as a difference from member 0)
    ctx.check(ctx.L.bbgpu_eval_upload(ctx.h, _lib.MC, B, sr.shape[2], _lib.ptr(sr), _lib.ptr(nv), _lib.ptr(descs)))
    ctx.check(ctx.L.bbgpu_eval_upload_profile(ctx.h, ms.shape[2], _lib.ptr(ms), _lib.ptr(L._prof["widx"]),
                                              _lib.ptr(L._prof["wval"])))
    ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
    nprof, mc_full, mc_delta, mc_replay = ctx.shared_members()
    alg = algorithmic(dm, L, sr, nv, descs, mc_full)
    # the longest of the MC model's and the convolution's stages that have a byte count: none of them runs on the
    # tensor pipes (integer and f32 FMA work), so the line is their HBM fraction; the ncu summaries in profiles/
    # give the pipes that bound them
    members = {"mc_deposit": mc_full, "mc_replay": mc_replay, "conv_resid": B}
    dom = max((k for k in members if k in kt and members[k]), key=kt.get)
    nbytes = alg[dom + "_bytes"](members[dom])
    achieved = nbytes / (kt[dom] * 1e-3) / 1e9
    used, tune = ctx.conv_variant()
    tkey = f"{dom}/{_lib.CONV_NAMES[used]}" if dom == "conv_resid" else dom
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": measured_traffic(tkey, B, members[dom]), "kernel": dom, "peak_source": src,
            "algorithmic_bytes": nbytes, "members": members[dom]}
    if dom == "conv_resid":
        # the convolution's useful arithmetic (2 x taps flop a voxel), and on the tensor cores its fraction of the
        # dense tensor peak (bf16 measured; tf32 runs at half that rate)
        useful = alg["conv_resid"][1] / (kt[dom] * 1e-3) / 1e12
        roof["conv_variant"] = _lib.CONV_NAMES[used]
        roof["useful_tflops"] = useful
        if used:
            tpk = bf16 if used == _lib.CONV_BF16X3 else bf16 / 2.
            roof["tensor"] = {"achieved_useful_tflops": useful, "peak_tflops": tpk, "frac": useful / tpk,
                              "peak": "bf16 dense (measured)" if used == 1 else "tf32 dense (half the measured bf16)"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": f"f32 models, {_lib.CONV_NAMES[used]} beam convolution, f64 reductions; bit-exact int cloud indices",
            "data": "synthetic",
            "config": {"workload": "global160: GLOBAL 3DFIT 160x160x128, 40 rings, MC GALMOD, 13x9 beam, batch of "
                                   f"{B} (base + 160 parameter steps)", "batch": B, "galmodtype": "MC",
                       "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (per-batch models 2 GB)",
                       "flux_normalisation": "deconvolved density profile recomputed at every evaluation (ring "
                                             "maps, beam, weighted NNLS with the smoothness prior), as the reference "
                                             "with DENS not fitted and the geometry free",
                       "shared": {"profiles_computed": nprof, "mc_members_full": mc_full,
                                  "mc_members_difference": mc_delta, "mc_members_replay": mc_replay,
                                  "note": "members equal to the first but for a few sub-rings are computed as its "
                                          "result plus the exact difference (bit-identical; 'unshared' below "
                                          "computes every member in full)"}},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "kernel_ms": kt, "roofline": roof, "clocks": clocks,
            "conv": {"variant": _lib.CONV_NAMES[used], "autotune_ms": tune},
            "graph": {"replays": graph_replays, "kernels_per_replay": graph_kernels,
                      "note": "the timed batch runs replay one CUDA graph of the batch (two streams, fork and join)"},
            "logL_sample": [float(out[0]), float(out[1])]}
    if not args.no_variants:
        line["conv"]["variants"] = conv_variants_leg(ctx, L, rows, rings, sr, nv, descs)
    if not args.no_analytic:
        line["analytic"] = analytic_leg(ctx, L, rows, rings, sr, nv, descs, args, dist, world)
    if B == 161 and not args.no_central:
        line["central_321"] = batch_leg(ctx, L, rings, step_rows(rings, 321), args, dist, world)
    if not args.no_random:
        line["random"] = batch_leg(ctx, L, rings, random_rows(rings, B), args, dist, world)
        line["unshared"] = batch_leg(ctx, L, rings, rows, args, dist, world, share=False)
    if not args.no_classic:
        line["classic_fit"] = classic_leg()
    if not args.no_ragged:
        line["ragged"] = ragged_leg(args, dist, world)
    if not args.no_wind:
        line["wind"] = wind_leg(args, dist, world, cpu=rank == 0 and not args.no_cpu)
    if not args.no_galwind:
        line["galwind"] = galwind_leg(args, dist, world, cpu=rank == 0 and not args.no_cpu)
    if not args.no_bayes:
        line["bayes256"] = bayes256_leg(args, dist, world, nb=args.bayes_nb)
        if not args.no_bayes_fit:
            line["bayes_fit"] = bayes_fit_leg()
    if rank == 0 and not args.no_cpu:
        vals, cores, n = cpu_leg(dm, L, rows, rings, data, mask)
        line["cpu_baseline"] = {"value": float(np.median(vals)), "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{n} evaluations of the batch, one per process (C restatement of the "
                                          "numba kernels + scipy FFT convolution)"}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def conv_variants_leg(ctx, L, rows, rings, sr, nv, descs):
    """Each variant of the batch convolution (float32, bf16x3 and tf32x3 on the tensor cores): its device time on the
    bench batch, and the largest relative error of a smoothed voxel (above 1e-6 of the peak) of two members against
    the float64 FFT convolution of the same model (scipy, the reference's algorithm in float64)."""
    from scipy.signal import fftconvolve
    from bbarolo2_gb300 import _lib
    dm = L.model
    B = rows.shape[0]
    ms = L._maps_sr                      # (the map tables of the whole batch: prepare() below replaces them)
    assert ms.shape[0] == B
    res = {}
    try:
        for v in (_lib.CONV_F32, _lib.CONV_BF16X3, _lib.CONV_TF32X3):
            ctx.set_option(_lib.OPT_CONV, v)
            ctx.check(ctx.L.bbgpu_eval_upload(ctx.h, _lib.MC, B, sr.shape[2], _lib.ptr(sr), _lib.ptr(nv),
                                              _lib.ptr(descs)))
            ctx.check(ctx.L.bbgpu_eval_upload_profile(ctx.h, ms.shape[2], _lib.ptr(ms), _lib.ptr(L._prof["widx"]),
                                                      _lib.ptr(L._prof["wval"])))
            ctx.set_option(_lib.OPT_TIMING, 1)
            t = []
            for _ in range(3):
                ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
                t.append(ctx.run_times()["conv_resid"])
            ctx.set_option(_lib.OPT_TIMING, 0)
            ctx.set_option(_lib.OPT_KEEP_SMOOTHED, 1)
            s2, n2, d2, b2 = L.prepare(rows[:2], rings, seed=1)
            L.run(s2, n2, d2)
            worst = 0.0
            for k, (blo, bhi) in enumerate(b2):
                by, bx, nz = bhi[1] - blo[1], bhi[0] - blo[0], L.shape[0]
                sm = np.zeros((by, bx, nz), np.float32)
                mo = np.zeros((by, bx, nz), np.float32)
                ctx.check(ctx.L.bbgpu_eval_model(ctx.h, k, 1, _lib.ptr(sm), by, bx, nz))
                ctx.check(ctx.L.bbgpu_eval_model(ctx.h, k, 0, _lib.ptr(mo), by, bx, nz))
                ref = fftconvolve(mo.astype(np.float64).transpose(2, 0, 1), dm.cfield[None], mode="same",
                                  axes=(1, 2)).transpose(1, 2, 0)
                ref[ref < 1e-12] = 0.
                ref *= dm.scalefactor
                big = ref > 1e-6 * ref.max()
                worst = max(worst, float((np.abs(sm[big] - ref[big]) / ref[big]).max()))
            ctx.set_option(_lib.OPT_KEEP_SMOOTHED, 0)
            res[_lib.CONV_NAMES[v]] = {"conv_ms": float(np.median(t)), "max_rel_err_vs_fp64": worst}
    finally:
        ctx.set_option(_lib.OPT_KEEP_SMOOTHED, 0)
        ctx.set_option(_lib.OPT_CONV, _lib.CONV_AUTO)
        L._maps_sr = ms                  # (the whole batch's tables, which the next legs upload)
    return res


def bayes256_leg(args, dist, world, nb=1024):
    """BAYESIAN 3DFIT at 256x256x192 (20 rings; VROT and VDISP per ring, INC and PA global: 42 dimensions; priors
    vrot 0-350 km/s, vdisp 1-40 km/s, inc 30-80, pa 0-360; truth drawn from them with seed 7; beam 4 pixels; noise 1%
    of the peak; the ANALYTIC model, the reference's default for BAYESIAN): one batch of nb independent points about
    the truth, as a nested sampler's live points late in a run, evaluated per launch (device-resident, the batch run
    replayed as a CUDA graph) and end to end. DENS is fixed at the truth (no flux normalisation)."""
    from bbarolo2_gb300 import _lib, bayesian, configs, engine
    cube, rings = configs.bayes256(galmodtype="ANALYTIC")
    dm = engine.DiskModel(cube, galmodtype="ANALYTIC")
    truth = dm.array(rings, seed=1)
    sigma = 0.01 * float(truth.max())
    g = np.random.default_rng(7)
    data = (truth + g.normal(0., sigma, truth.shape)).astype(np.float32)
    L = engine.BatchLikelihood(dm, data, truth > 3 * sigma, maskmode=2, sigma=sigma)
    prob = bayesian.Problem(rings, per_ring=("vrot", "vdisp"), global_=("inc", "phi"),
                            priors={"vrot": (0., 350.), "vdisp": (1., 40.), "inc": (30., 80.), "phi": (0., 360.)})
    t0 = np.clip(prob.unit(np.r_[rings.vrot, rings.vdisp, rings.inc[0], rings.phi[0]])[0], 0, 1)
    ctx = dm.ctx
    while True:
        u = np.clip(t0 + 0.002 * g.standard_normal((nb, prob.ndim)), 0., 1.)
        rows = prob.rows(u)
        try:
            sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
            ctx.check(ctx.L.bbgpu_eval_upload(ctx.h, _lib.ANALYTIC, nb, sr.shape[2], _lib.ptr(sr), _lib.ptr(nv),
                                              _lib.ptr(descs)))
            ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
            break
        except _lib.DeviceError:
            if nb <= 128:
                raise
            nb //= 2                   # (device memory: halve the batch)
    steps = max(2, args.steps // 4)
    for _ in range(2):
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
    ctx.check(ctx.L.bbgpu_sync(ctx.h))
    t = time.perf_counter()
    for _ in range(steps):
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
    ctx.check(ctx.L.bbgpu_sync(ctx.h))
    dt = max_over_ranks(time.perf_counter() - t, dist)
    replays, kernels = ctx.graph_stats()
    ctx.set_option(_lib.OPT_TIMING, 1)
    ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
    kt = {k: round(v, 3) for k, v in ctx.run_times().items() if v > 0.01}
    ctx.set_option(_lib.OPT_TIMING, 0)
    L.evaluate(rows, rings, seed=1, galmodtype="ANALYTIC")
    t = time.perf_counter()
    for _ in range(steps):
        L.evaluate(rows, rings, seed=1, galmodtype="ANALYTIC")
    te = max_over_ranks(time.perf_counter() - t, dist)
    return {"batch": nb, "ndim": prob.ndim, "value": throughput(nb, steps, world, dt), "unit": UNIT,
            "ms_per_step": 1e3 * dt / steps, "e2e": throughput(nb, steps, world, te), "kernel_ms": kt,
            "graph": {"replays": replays, "kernels_per_replay": kernels},
            "config": "256x256x192, 20 rings, 42 dimensions, ANALYTIC, DENS fixed"}


def bayes_fit_leg(seed=11):
    """BAYESIAN fit time at dlogZ <= 0.1 (nested sampling, 100 live points, batches of 1024 proposals) on the
    256x256x192 cube of the BAYESIAN workload (20 rings, ANALYTIC) with VROT and VDISP of four rings free (8
    dimensions; ``configs.bayes256_subproblem``): plain, then with the learned surrogate screening the proposals (same
    seed: the same proposals)."""
    from bbarolo2_gb300 import bayesian, configs
    like, prob = configs.bayes256_subproblem()
    kw = dict(n_live=100, n_batch=1024, dlogz=0.1, seed=seed, galmodtype="ANALYTIC")
    out = {}
    for name, sur in (("plain", False), ("screened", True)):
        res = bayesian.fit(like, prob, surrogate=sur, **kw)
        out[name] = {"wall_s": res["wall"], "logz": res["logz"], "logzerr": res["logzerr"], "n_like": res["n_like"],
                     "n_proposed": res["n_proposed"], "iterations": res["iterations"]}
        if sur:
            out[name].update(n_screened=res["n_screened"], screen_batches=res["screen_batches"],
                             surrogate_rmse=res.get("surrogate_rmse"))
        out[name]["theta_median"] = [round(float(v), 4) for v in res["theta_median"]]
        out[name]["theta_std"] = [round(float(v), 4) for v in res["theta_std"]]
    sd = np.asarray(out["plain"]["theta_std"])
    out["dlogz_screened_vs_plain"] = out["screened"]["logz"] - out["plain"]["logz"]
    out["max_median_shift_sigma"] = float(np.max(np.abs(np.asarray(out["screened"]["theta_median"]) -
                                                      np.asarray(out["plain"]["theta_median"])) / sd))
    out["speedup"] = out["plain"]["wall_s"] / out["screened"]["wall_s"]
    out["calls_ratio"] = out["plain"]["n_like"] / out["screened"]["n_like"]
    out["problem"] = "256x256x192, 20 rings, VROT+VDISP of 4 rings free (8 dimensions), ANALYTIC, 100 live points"
    return out


def classic_leg():
    """CLASSIC 3DFIT of the 64x64x64 workload (8 rings, VROT and VDISP free from 120 and 8 km/s, the reference's
    defaults: NORM AZIM, FTYPE 2, WFUNC 2; noise 1% of the peak, seed 1; mask of the model above three times the
    noise): the fit's wall time (the rings of the stage advanced together, each evaluation a single-ring model,
    sparse convolution and normalisation on the device), its evaluations, and the fitted values against the truth."""
    from bbarolo2_gb300 import classic, configs, engine
    cube, rings = configs.classic64(galmodtype="MC")
    dm = engine.DiskModel(cube)
    truth = dm.array(rings, seed=1)
    sigma = 0.01 * float(truth.max())
    g = np.random.default_rng(1)
    cube.array = (truth + g.normal(0., sigma, truth.shape)).astype(np.float32)
    inr = rings.copy()
    inr.vrot = np.full(inr.nr, 120.)
    inr.vdisp = np.full(inr.nr, 8.)
    fit = classic.ClassicFit(cube, inr, classic.default_par(), sigma, truth > 3 * sigma)
    fit.run()                                  # (warm-up: device buffers and the rings' cloud layouts)
    fit = classic.ClassicFit(cube, inr, classic.default_par(), sigma, truth > 3 * sigma)
    t = time.perf_counter()
    out, ok = fit.run()
    wall = time.perf_counter() - t
    n = sum(len(v) for v in fit.log.values())
    return {"wall_s": wall, "evaluations": n, "ms_per_evaluation": 1e3 * wall / max(n, 1),
            "rings_converged": int(sum(ok)), "rings": int(rings.nr),
            "max_abs_err_vrot": float(np.max(np.abs(out.vrot - rings.vrot))),
            "max_abs_err_vdisp": float(np.max(np.abs(out.vdisp - rings.vdisp))),
            "problem": "64x64x64, 8 rings, VROT+VDISP free from 120/8 km/s, MC model, one stage"}


def ragged_leg(args, dist, world, ngal=128, nb=4):
    """A heterogeneous batch (``ragged.GalaxyBatch``): ngal galaxies of the heterogeneous population (seed 11: cubes
    of 32-320 pixels a side and 32-256 channels, 5-50 rings, every geometry, scale height and beam different; the
    ANALYTIC model), nb ring sets about each galaxy's truth; every galaxy's batch queued on its own context and
    stream before any result is read, graph replays once warm. Device rate (upload once, runs and result reads
    timed) and end to end (ring tables, uploads, runs and reads timed)."""
    from bbarolo2_gb300 import configs
    from bbarolo2_gb300.galmod import ring_rows_batch
    from bbarolo2_gb300.ragged import GalaxyBatch
    pop = configs.galaxy_population(ngal, seed=11)
    batch = GalaxyBatch.mock(pop, seed=3)
    g = np.random.default_rng(5)
    rows = []
    for _, _, rings in batch.items:
        r = ring_rows_batch([rings] * nb)
        r[1:, 4] *= 1 + 0.02 * g.standard_normal((nb - 1, rings.nr))
        r[1:, 5] *= 1 + 0.05 * g.random((nb - 1, rings.nr))
        rows.append(r)
    boxes = batch.upload(rows, seed=1)
    for _ in range(3):
        batch.run()
        batch.download(boxes)
    steps = max(2, args.steps // 2)
    t = time.perf_counter()
    for _ in range(steps):
        batch.run()
        batch.download(boxes)
    dt = max_over_ranks(time.perf_counter() - t, dist)
    t = time.perf_counter()
    for _ in range(steps):
        batch.evaluate(rows, seed=1)
    te = max_over_ranks(time.perf_counter() - t, dist)
    n = ngal * nb
    vox = [c.DimX() * c.DimY() * c.DimZ() for c, _, _ in pop]
    return {"galaxies": ngal, "per_galaxy": nb, "value": throughput(n, steps, world, dt), "unit": UNIT,
            "ms_per_step": 1e3 * dt / steps, "e2e": throughput(n, steps, world, te),
            "voxels_per_cube": {"min": int(min(vox)), "median": int(np.median(vox)), "max": int(max(vox))},
            "note": "one context and stream per galaxy, all queued before the reads; not one launch"}


def wind_leg(args, dist, world, cpu=True):
    """WINDFIT's per-likelihood column work on the Circinus-shaped problem (``configs.wind_circinus``: 3192 cells,
    1.9 million quadrature points, 173x238x41 voxels): for one wind, the quadrature points, the columns (deposit and
    beam convolution) and the normal equations G, b of the columns over the voxel lists pruned at 1e-3 (the default
    of the reference's likelihood), G (3192 x 3192) and b read back. Each step a new wind (VWIND and INC moved, as a
    fit moves them), through the public API (``WindModel.boxes``, ``Boxes.voxel_lists``, ``Boxes.normal``). The CPU
    leg: the oracle (the reference's kernels restated in C, one thread) on one wind; parity: its G and b against
    the device's."""
    from bbarolo2_gb300 import configs
    from bbarolo2_gb300.wind import WindPars
    wm, p0 = configs.wind_circinus()
    W, Wd = configs.wind_data(wm, p0)
    rel = 1e-3

    def wind(k):
        return WindPars(p0.radii, p0.vwind + 3. * (k % 7), 0., xpos=p0.xpos, ypos=p0.ypos, inc=p0.inc + 0.05 * (k % 5),
                        pa=p0.pa, openang=p0.openang, conelen=p0.conelen)

    def one(k, stages=None):
        t0 = time.perf_counter()
        B = wm.boxes(wind(k))
        t1 = time.perf_counter()
        G, b = B.normal(Wd, W, B.voxel_lists(W, rel=rel))
        if stages is not None:
            stages[0] += t1 - t0
            stages[1] += time.perf_counter() - t1
        return B, G, b

    for k in range(max(3, args.warmup)):
        one(k)
    steps = max(3, args.steps // 2)
    stages = [0., 0.]
    l0 = wm.launches()
    t = time.perf_counter()
    for k in range(steps):
        B, G, b = one(k, stages)
    dt = max_over_ranks(time.perf_counter() - t, dist)
    launches = (wm.launches() - l0) // steps
    out = {"workload": "wind_circinus: 173x238x41 voxels, 3192 cells (approaching cone), "
                       f"{wm.cells.npoints} quadrature points, beam kernel {2 * wm.hy + 1}x{2 * wm.hx + 1}",
           "metric": "wind likelihood column evaluations/s (points + columns + normal equations, G and b read)",
           "value": throughput(1, steps, world, dt), "ms_per_evaluation": 1e3 * dt / steps,
           "ms_columns": 1e3 * stages[0] / steps, "ms_normal": 1e3 * stages[1] / steps,
           "column_values": int(B.total), "nonempty_columns": int(np.sum(np.diff(B.offs) > 0)),
           "gpu_launches_per_evaluation": int(launches), "prune": rel,
           "d2h_bytes_per_evaluation": int(G.nbytes + b.nbytes + B.boxes.nbytes)}
    if cpu:
        from oracle import oracle as O
        p = wind(steps - 1)
        su = wm.setup
        inc, ang = math.radians(p.inc), math.radians(p.pa) + su.crota2
        t = time.perf_counter()
        pts = O.wind_points(wm.cells.cells, wm.cells.qn, wm.cells.qoff, p.radii, p.vwind, p.vdisp, p.vrot, p.xpos,
                            p.ypos, p.vsys * 1000., math.sin(inc), math.cos(inc), math.sin(ang), math.cos(ang),
                            wm.cdelt[0], wm.cdelt[1], math.radians(0.5 * p.openin), math.radians(0.5 * p.openang),
                            p.conelen, su.sig_instr)
        spec = dict(chmin=su._chmin, axtyp=su.axtyp, velsys=su.velsys, lfreq0=su.lfreq0, crval3=su.crval3,
                    cdelt3=su.cdelt3, crpix3=su.crpix3)
        nz, ny, nx = wm.shape
        lim = np.array([0, nx, 0, ny, 0, nz])
        buf, offs, boxes = O.wind_boxes(pts, pts["w"], lim, wm.shape, wm.kern, wm.kx, wm.ky, wm.separable, spec,
                                        su._vedges_lines, su.relint, wm.cells.qoff)
        Go, bo = O.wind_normal(buf, offs, boxes, Wd, W, lim, rel)
        tc = time.perf_counter() - t
        out["cpu_baseline"] = {"value": 1. / tc, "unit": "evaluations/s", "cores": 1, "kind": "port",
                               "sample": "one wind: the oracle's points, columns and normal equations"}
        out["max_rel_err_G"] = float(np.abs(G - Go).max() / np.abs(Go).max())
        out["max_rel_err_b"] = float(np.abs(b - bo).max() / np.abs(bo).max())
        out["boxes_equal"] = bool(np.array_equal(B.boxes, boxes))
    wm.close()
    return out


def galwind_leg(args, dist, world, cpu=True):
    """GALWIND WTYPE 1 (the Monte-Carlo shells of a bi-cone, ``galwind.GalWindMC``) on a 128x128x64 cube of 4"
    pixels and 10 km/s channels: CONELEN 240" (80 shells 3" apart), OPENANG 60, VWIND 300, VDISP 20 km/s, DENS 10,
    CDENS 20, NV 20, INC 60, PHI 45, 16 chunks of shells (THREADS 16): the model's wall time through the public API
    (streams parsed on host threads, clouds placed and deposited on the device, the cube read back). The CPU leg: the
    oracle (the reference's _galmod_wind restated in C, one thread) over the same chunks; parity: the two models."""
    from bbarolo2_gb300.cube import Cube, Params
    from bbarolo2_gb300.galwind import GalWindMC, GalWindPars
    cube = Cube.empty(128, 128, 64, [-4. / 3600., 4. / 3600., 10.], par=Params(), crpix=[64.5, 64.5, 32.5],
                      crval=[60., 0., 0.], cunit=("deg", "deg", "km/s"))
    par = GalWindPars(xpos=63.5, ypos=63.5, vsys=0., inc=60., phi=45., conelen=240., nlayers=30, vwind=300.,
                      vdisp=20., dens=10., openang=60., cdens=20., nv=20, iseed=3)
    gw = GalWindMC(cube, par, threads=16)
    for _ in range(max(2, args.warmup)):
        mod = gw.model()
    steps = max(3, args.steps // 4)
    t = time.perf_counter()
    for _ in range(steps):
        mod = gw.model()
    dt = max_over_ranks(time.perf_counter() - t, dist)
    st = gw.setup
    nc = np.rint(st.cdens * gw.sr[4] * 2 * math.pi * gw.sr[0] * gw.sep / st.pixarea)
    out = {"workload": "galwind_shells: 128x128x64 voxels, %d shells, %d clouds, %d velocity samples, 16 chunks"
                       % (gw.sr.shape[1], int(nc.sum()), int((nc * gw.nv).sum())),
           "metric": "GALWIND WTYPE 1 models/s (streams parsed, clouds deposited, cube read back)",
           "value": throughput(1, steps, world, dt), "ms_per_model": 1e3 * dt / steps}
    if cpu:
        from oracle import oracle as O
        ref = np.zeros((cube.DimY(), cube.DimX(), cube.DimZ()))
        seed = int(par.ISEED) & 0xFFFFFFFF
        t = time.perf_counter()
        for k, ch in enumerate(gw.chunks()):
            ref += O.galmod_wind(np.zeros_like(ref), gw.sr, int(ch[0]), int(ch[-1]) + 1,
                                 (seed + 7919 * k) & 0xFFFFFFFF, gw.sep, gw.nv, st.cdens, 1, st.pixarea, st.cdelt[0],
                                 st.cdelt[1], st.crota2, 0, 0, cube.DimX(), cube.DimY(), st.sig_instr, st.axtyp,
                                 st.velsys, st.lfreq0, st.crval3, st.cdelt3, st.crpix3, st.relint, st.cd2i)
        tc = time.perf_counter() - t
        ref = ref.transpose(2, 0, 1)
        out["cpu_baseline"] = {"value": 1. / tc, "unit": "models/s", "cores": 1, "kind": "port",
                               "sample": "one model: the oracle's _galmod_wind over the 16 chunks"}
        out["same_voxels"] = bool(np.array_equal(mod != 0, ref != 0))
        out["max_rel_err"] = float(np.max(np.abs(mod - ref) / np.maximum(np.abs(ref), 1e-300)))
    return out


def random_rows(rings, batch, seed=2):
    """Ring-value rows of independent points about the base point, as nested-sampling live points: every member
    moves VROT, VDISP, INC and PA of every ring (uniform within 5 km/s, 1 km/s, 1 and 1 degree), so that no two
    members share a ring map."""
    base = ring_rows(rings)
    rows = np.repeat(base[None], batch, axis=0)
    g = np.random.default_rng(seed)
    for row, half in ((4, 5.0), (5, 1.0), (12, 1.0), (13, 1.0)):
        rows[1:, row, :] += g.uniform(-half, half, (batch - 1, rings.nr))
    return rows


def batch_leg(ctx, L, rings, rows, args, dist, world, share=True):
    """Another batch of the same problem (MC): device-resident evaluations/s and end to end. share=False
    computes every member's flux normalisation from all its samples (no member shares member 0's ring maps)."""
    from bbarolo2_gb300 import _lib
    ctx.set_option(_lib.OPT_SHARE, 1 if share else 0)
    try:
        sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
        B = rows.shape[0]
        steps = max(1, args.steps // 2)
        ctx.check(ctx.L.bbgpu_eval_upload(ctx.h, _lib.MC, B, sr.shape[2], _lib.ptr(sr), _lib.ptr(nv),
                                          _lib.ptr(descs)))
        ms = L._maps_sr
        ctx.check(ctx.L.bbgpu_eval_upload_profile(ctx.h, ms.shape[2], _lib.ptr(ms), _lib.ptr(L._prof["widx"]),
                                                  _lib.ptr(L._prof["wval"])))
        for _ in range(args.warmup):
            ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
        ctx.check(ctx.L.bbgpu_sync(ctx.h))
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
        ctx.check(ctx.L.bbgpu_sync(ctx.h))
        dt = max_over_ranks(time.perf_counter() - t0, dist)
        ctx.set_option(_lib.OPT_TIMING, 1)
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
        kt = {k: round(v, 4) for k, v in ctx.run_times().items() if k.startswith("prof_")}
        ctx.set_option(_lib.OPT_TIMING, 0)
        L.evaluate(rows, rings, seed=1)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            L.evaluate(rows, rings, seed=1)
        te = max_over_ranks(time.perf_counter() - t0, dist)
    finally:
        ctx.set_option(_lib.OPT_SHARE, 1)
    return {"batch": B, "value": throughput(B, steps, world, dt), "unit": UNIT, "steps": steps,
            "ms_per_step": 1e3 * dt / steps, "e2e": throughput(B, steps, world, te), "profile_ms": kt}


def analytic_leg(ctx, L, rows, rings, sr, nv, descs, args, dist, world):
    """The same batch with the ANALYTIC GALMOD (the reference's default for GLOBAL): device-resident evaluations/s,
    the stage times, and end to end through the Python API."""
    from bbarolo2_gb300 import _lib
    B = rows.shape[0]
    steps = max(1, args.steps // 2)
    ctx.check(ctx.L.bbgpu_eval_upload(ctx.h, _lib.ANALYTIC, B, sr.shape[2], _lib.ptr(sr), _lib.ptr(nv),
                                      _lib.ptr(descs)))
    ms = L._maps_sr
    ctx.check(ctx.L.bbgpu_eval_upload_profile(ctx.h, ms.shape[2], _lib.ptr(ms), _lib.ptr(L._prof["widx"]),
                                              _lib.ptr(L._prof["wval"])))
    for _ in range(args.warmup):
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
    ctx.check(ctx.L.bbgpu_sync(ctx.h))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
    ctx.check(ctx.L.bbgpu_sync(ctx.h))
    dt = max_over_ranks(time.perf_counter() - t0, dist)
    ctx.set_option(_lib.OPT_TIMING, 1)
    ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
    kt = {k: v for k, v in ctx.run_times().items() if v > 0}
    ctx.set_option(_lib.OPT_TIMING, 0)
    L.evaluate(rows, rings, seed=1, galmodtype="ANALYTIC")
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        out = L.evaluate(rows, rings, seed=1, galmodtype="ANALYTIC")
    te = max_over_ranks(time.perf_counter() - t0, dist)
    return {"value": throughput(B, steps, world, dt), "unit": UNIT, "steps": steps, "ms_per_step": 1e3 * dt / steps,
            "e2e": throughput(B, steps, world, te), "kernel_ms": kt, "logL_sample": [float(out[0]), float(out[1])]}


def reference_arm(args, world):
    """The reference's CPU evaluation of the same workload on the host cores, with the oracle alone: the
    reference's host set-up restated in ``oracle/host.py``, its numba kernels restated in C (``oracle/bbref.c``),
    its FFT convolution and profile solve with scipy (``oracle/cpu_baseline.py``); one evaluation per process on
    every host core, as the reference's process pool. Each step evaluates the whole batch (the same members as
    the device arm); the ANALYTIC model and the batch of independent points are timed on bounded samples. The
    product library is not loaded."""
    from bbarolo2_gb300 import configs           # the workload's definition (header values and rings)
    from oracle import cpu_baseline as CB
    cube, rings = configs.global160(galmodtype="MC")
    rows = step_rows(rings, args.batch)
    B = rows.shape[0]
    pool = CB.Pool(CB.reference_payload(cube, rings, rows))
    cores = pool.cores
    for _ in range(max(1, min(args.warmup, 2))):
        pool.run(range(B))
    t = 0.0
    for _ in range(args.steps):
        t += pool.run(range(B))[1]
    pool.close()
    v = B * args.steps / t
    legs = {}
    for name, galmodtype, rws, n in (("analytic", "ANALYTIC", rows, min(B, 2 * cores)),
                                     ("random", "MC", random_rows(rings, B), min(B, 4 * cores))):
        pool = CB.Pool(CB.reference_payload(cube, rings, rws, galmodtype=galmodtype))
        pool.run(range(min(n, cores)))
        _, wall = pool.run(range(n))
        pool.close()
        legs[name] = {"value": n / wall, "unit": UNIT, "sample": f"{n} evaluations of the batch, one per process"}
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "global160: GLOBAL 3DFIT 160x160x128, 40 rings, MC GALMOD, 13x9 beam, batch of "
                                   f"{B} (base + 160 parameter steps)", "batch": B, "galmodtype": "MC",
                       "parallelism": f"{cores} host processes"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{B} evaluations per step (the whole batch), one per process: the reference's "
                                       "host set-up, C restatement of its numba kernels, scipy FFT convolution and "
                                       "NNLS"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line.update(legs)
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
