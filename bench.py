"""Benchmark of the periodic-box bispectrum on GB300.

Workload (the headline metric): ``compute_bispec_in_gpp_box``, B_000 diag,
20 linear bins 0.005-0.205 h/Mpc, 4 194 304 particles uniform in a
1000 Mpc/h box (numpy ``default_rng(42)``, float64), unit weights,
nz = N/V, 512^3 mesh, TSC, no interlacing (three-point statistics force it
off), particle normalisation.  One step = one estimate.

Lines printed by rank 0 (one JSON object):
  value  -- s/estimate of the FP32-mixed path with particles resident in
            device memory (CUDA events on the stream the library runs on);
  e2e    -- the same through the C ABI with pinned host particle arrays,
            host->device copies inside the timed region;
  fp64   -- the FP64 path on the same inputs, its time and the FP32-mixed
            per-bin error against it;
  b202_diag -- B_202 diag on the same catalogue (FP32-mixed and FP64);
  oracle_check -- the FP32-mixed and FP64 estimates against the CPU
            oracle's own values of two bins at the full workload size;
  cold_first_call_s -- the first estimate of a fresh context;
  roofline, cpu_baseline, clocks, gpu_launches.
Step times are the median of the timed steps.
``--impl reference`` times the CPU oracle (a numpy restatement of the
reference algorithm) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("bispectrum s/estimate @512³, 4M pts: FP32-mixed vs FP64 on "
          "1 GB300 @1e-5 err")
UNIT = "s/estimate"
FALLBACK_HBM_GBS = 6800.


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--ngrid', type=int, default=512)
    ap.add_argument('--npart', type=int, default=4194304)
    ap.add_argument('--boxsize', type=float, default=1000.)
    ap.add_argument('--nbins', type=int, default=20)
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-fp64', action='store_true')
    ap.add_argument('--no-b202', action='store_true',
                    help='skip the B_202 diag timing and error')
    ap.add_argument('--profile-only', action='store_true',
                    help='run two estimates (for an ncu launch list; with '
                         '--workload survey two B_202 estimates)')
    ap.add_argument('--variants', action='store_true',
                    help='also time the FP32-mixed precision options')
    ap.add_argument('--workload', default='metric',
                    choices=['metric', 'mocks', 'survey', 'large'],
                    help="'mocks': the batched lognormal-mock workload; "
                         "'survey': survey bispectra from device "
                         "catalogues; 'large': the 1024^3 lognormal box "
                         "(bispectra full 40x40, 3PCF on 30 bins); each "
                         "prints its own JSON line")
    ap.add_argument('--mocks', type=int, default=256)
    ap.add_argument('--mesh-comp', type=int, default=2, choices=[0, 1, 2],
                    help='compensated FP32 mesh deposit (library option '
                         '"mesh_comp")')
    ap.add_argument('--side-priority', type=int, default=0, choices=[0, 1],
                    help='priority of the second stream (library option '
                         '"side_priority")')
    ap.add_argument('--seed', type=int, default=42,
                    help='seed of the uniform catalogue (metric workload)')
    ap.add_argument('--ff-transforms', type=int, default=1, choices=[0, 1, 2],
                    help='float-float transforms of the shell fields: 1 both '
                         'directions, 2 the forward transform only, 0 none '
                         '(library option "ff_transforms")')
    ap.add_argument('--assign-path', type=int, default=0, choices=[0, 1, 2],
                    help='deposit of sorted catalogues: 0 autotuned, '
                         '1 shared-memory tiled, 2 per-particle atomics')
    return ap.parse_args()


def workload(args):
    return {
        "workload": (f"gpp B_000 diag, {args.ngrid}^3 mesh, TSC, "
                     f"{args.npart} uniform particles, L={args.boxsize:g} "
                     f"Mpc/h, {args.nbins} lin k-bins 0.005-0.205 h/Mpc"),
        "ngrid": args.ngrid, "npart": args.npart, "boxsize": args.boxsize,
        "bins": [0.005, 0.205, args.nbins], "assignment": "tsc",
        "degrees": [0, 0, 0], "form": "diag", "norm": "particle",
        "l2": ("inputs larger than L2 (mesh >= 512 MiB) and a 256 MiB L2 "
               "flush before every timed step"),
    }


def make_particles(n, box, seed=42):
    rng = np.random.default_rng(seed)
    x, y, z = rng.uniform(0., box, size=(3, n))
    # ParticleCatalogue.periodise (catalogue.py:648-676), as the Python
    # entry point does before handing positions to the estimator.
    out = []
    for c in (x, y, z):
        out.append(np.ascontiguousarray(
            (c + box / 2. - (c.max() + c.min()) / 2.) % box))
    return out


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed
    region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.device),
                 f'--query-gpu={self.QUERY}', '--format=csv,noheader,nounits',
                 '-lms', '200'], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown',
                 'sw_power_cap']
        for ln in self.lines:
            f = [v.strip() for v in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary."""
    f = ROOT / "profiles" / "ncu_traffic.json"
    if not f.exists():
        return None
    try:
        return json.loads(f.read_text()).get(kernel)
    except ValueError:
        return None


def good_fft_size(n):
    """Smallest 2^a 3^b 5^c >= n (the evaluation-grid size rule)."""
    while True:
        m = n
        for f in (2, 3, 5):
            while m % f == 0:
                m //= f
        if m == 1:
            return n
        n += 1


def band_half_width(args):
    """Largest |s| of a shell mode of the workload (k < kmax)."""
    kmax = getattr(args, 'kmax', 0.205)
    return int(np.floor(kmax / (2 * np.pi / args.boxsize))) + 1


def eval_grid(args):
    """Evaluation-grid size M of the workload's shells (k < kmax)."""
    return min(args.ngrid, good_fft_size(4 * band_half_width(args) + 1))


def algorithmic_bytes(kernel, args, real_bytes):
    """Compulsory HBM bytes of one launch of `kernel` on the FP32-mixed
    workload (every input read once, every output written once)."""
    nm = args.ngrid ** 3
    nh = args.ngrid * args.ngrid * (args.ngrid // 2 + 1)
    c = 2 * real_bytes          # complex value
    M = eval_grid(args)
    mc, mh = M ** 3, M * M * (M // 2 + 1)
    nkeys = 3 * (args.ngrid // 2) ** 2 + 1
    N, K = args.ngrid, band_half_width(args)
    Kg = 2 * K
    f4 = 16                     # float-float complex value

    def inv(nf, k):
        """Bytes of the three inverse passes of nf fields of band k."""
        x = 2 * f4 * nf * (k + 1) * (2 * k + 1) * M
        y = f4 * nf * (k + 1) * M * ((2 * k + 1) + M)
        z = f4 * nf * M * M * (k + 1) + 8 * nf * mc
        return x, y, z

    # Inverse launches per estimate: G (one field, band 2K) and the nbins
    # shell fields (band K); the per-launch figure is their mean.
    ig, i_f = inv(1, Kg), inv(args.nbins, K)
    table = {
        # float-float mesh transforms: the FP32 mesh read, z-pass spectrum
        # rows (kz <= 2K) written, and the FP32 planes of every row's z
        # transform (8 B per half-spectrum mode) that complete the mesh's
        # R2C; then the kept y and x bands.
        'ff_fwd_z_kernel': real_bytes * nm + f4 * N * (Kg + 1) * N + c * nh,
        # the planes read and the R2C-layout spectrum written.
        'planes_to_half_kernel': 2 * c * nh,
        'ff_fwd_y_kernel': f4 * N * (Kg + 1) * (N + 2 * Kg + 1),
        'ff_fwd_x_kernel': f4 * (2 * Kg + 1) * (Kg + 1) * (N + 2 * Kg + 1),
        'ff_inv_x_kernel': (ig[0] + i_f[0]) / 2,
        'ff_inv_y_kernel': (ig[1] + i_f[1]) / 2,
        'ff_inv_z_kernel': (ig[2] + i_f[2]) / 2,
        # shot-noise field xi read once; the key histogram written once.
        'orbit_rows_kernel': real_bytes * nm + 16 * nkeys,
        # G and the nbins shell fields (real, on M^3, float-float hi and lo
        # words) read once.
        'reduce_pairs_kernel': 2 * real_bytes * mc * (1 + args.nbins),
        # key histogram read once.
        'pair_bessel_sums_kernel': 16 * nkeys,
        # nbins half-spectrum shell fields on the evaluation grid written.
        'build_F_kernel': c * mh * args.nbins,
        # every mesh cell written once.
        'fill_offset_kernel': real_bytes * nm,
        # x, y, z read; every mesh cell written once.
        'assign_kernel': 24 * args.npart + real_bytes * nm,
        # x, y, z read; tile key and rank written.
        'tile_key_kernel': 32 * args.npart,
        # x, y, z, key, rank read; sorted x, y, z written.
        'scatter_kernel': 56 * args.npart,
        # half spectrum read, shot-noise half spectrum written.
        'twopt_field_kernel': 2 * c * nh,
        # shot-noise field read once.
        'radial_hist_kernel': real_bytes * nm,
        'cufft.r2c.mesh': real_bytes * nm + c * nh,
        'cufft.c2r.xi': c * nh + real_bytes * nm,
    }
    return table.get(kernel)


def run_gb300(args):
    import torch

    from triumvirate_gb300 import _engine, _lib
    from triumvirate_gb300.dataobjs import Binning

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=torch.device('cuda', local))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    box, n, N = args.boxsize, args.npart, args.ngrid
    x, y, z = make_particles(n, box, seed=args.seed + rank)
    binning = Binning('fourier', 'lin', 0.005, 0.205, args.nbins)
    nbar = n / box ** 3
    norm = 1. / (n * nbar ** 2)        # threept.cpp:96-136, alpha = 1

    ctx = _lib.Context(local)
    ctx.set_option('assign_path', args.assign_path)
    ctx.set_option('mesh_comp', args.mesh_comp)
    ctx.set_option('ff_transforms', args.ff_transforms)
    ctx.set_option('side_priority', args.side_priority)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)

    def params(precision, degrees=(0, 0, 0)):
        pd = {'boxsize': {'x': box, 'y': box, 'z': box},
              'ngrid': {'x': N, 'y': N, 'z': N}, 'assignment_order': 3,
              'interlace': False,
              'degrees': dict(zip(('ell1', 'ell2', 'ELL'), degrees)),
              'form': 'diag', 'shape': 'diag', 'precision': precision,
              'verbose': 0}
        return _engine.make_params(pd, '3pt')

    p32, p64 = params('fp32mixed'), params('fp64')
    xd, yd, zd = (torch.from_numpy(a).to(dev) for a in (x, y, z))
    dcat = _engine.device_catalogue(n, xd.data_ptr(), yd.data_ptr(),
                                    zd.data_ptr())
    xh, yh, zh = (torch.from_numpy(a).pin_memory() for a in (x, y, z))
    hcat = _engine.device_catalogue(n, xh.data_ptr(), yh.data_ptr(),
                                    zh.data_ptr())
    hcat.memory = _lib.MEM_HOST
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32,
                        device=dev)

    def estimate(p, cat):
        return _engine.call_threept('trvg_compute_bispec_in_gpp_box', ctx, p,
                                    cat, binning, norm, 'bispec',
                                    shape='diag')

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed(p, cat, steps, profile=False):
        ctx.set_option('profiling', int(profile))
        ms, launches, ktimes, res = [], 0, {}, None
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            barrier()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = estimate(p, cat)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms.append(e0.elapsed_time(e1))
            st = ctx.stats()
            launches += st['kernel_launches']
            if profile:
                for k, (t, c) in ctx.kernel_times().items():
                    a = ktimes.setdefault(k, [0., 0])
                    a[0] += t
                    a[1] += c
        ctx.set_option('profiling', 0)
        return ms, launches, ktimes, res, st

    if args.profile_only:
        for _ in range(2):
            estimate(p32, dcat)
        torch.cuda.synchronize(dev)
        return

    for _ in range(args.warmup):
        estimate(p32, dcat)
    estimate(p32, hcat)

    clocks = ClockSampler(local)
    clocks.start()
    ms, launches, _, res32, st = timed(p32, dcat, args.steps)
    clk = clocks.stop()
    ms_e2e, _, _, _, st_e2e = timed(p32, hcat, args.steps)
    # Per-kernel CUDA-event times from separate profiled estimates.
    nprof = 2
    _, _, ktimes, _, _ = timed(p32, dcat, nprof, profile=True)

    # Median step time per rank, then the maximum over ranks; the ranks
    # run their estimates side by side, so the job finishes `world`
    # estimates per such step.
    med_s = statistics.median(ms) / 1e3
    med_e2e = statistics.median(ms_e2e) / 1e3
    total_s = sum(ms) / 1e3
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([med_s, med_e2e, total_s], device=dev,
                         dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        med_s, med_e2e, total_s = float(t[0]), float(t[1]), float(t[2])
    value = med_s / world
    value_e2e = med_e2e / world

    # First estimate of a fresh context: FFT plans, autotuning trials,
    # spline / shell / statistics tables and workspace (the process has
    # already initialised CUDA and loaded the library).
    cold = _lib.Context(local)
    cold.set_option('assign_path', args.assign_path)
    cold.set_option('mesh_comp', args.mesh_comp)
    cold.set_option('ff_transforms', args.ff_transforms)
    cold.set_option('side_priority', args.side_priority)
    cold.set_stream(stream.cuda_stream)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    _engine.call_threept('trvg_compute_bispec_in_gpp_box', cold, p32, dcat,
                         binning, norm, 'bispec', shape='diag')
    torch.cuda.synchronize(dev)
    cold_first_call_s = time.perf_counter() - t0
    del cold

    fp64 = None
    res64 = None
    if not args.no_fp64:
        estimate(p64, dcat)
        n64 = max(1, min(args.steps, 3))
        ms64, _, _, res64, _ = timed(p64, dcat, n64)
        fp64 = {"s_per_estimate": statistics.median(ms64) / 1e3,
                "fp32mixed_speedup": statistics.median(ms64) /
                statistics.median(ms),
                "max_rel_err_fp32mixed": per_bin_err(res32, res64),
                "nmodes_equal": bool(np.array_equal(res32['nmodes_1'],
                                                    res64['nmodes_1']))}
        ctx.set_option('full_mesh_shells', 1)
        try:
            estimate(p64, dcat)
            msd, _, _, resd, _ = timed(p64, dcat, 1)
            fp64["plain_full_mesh_s_per_estimate"] = sum(msd) / 1e3
            fp64["fp32mixed_speedup_vs_plain"] = sum(msd) / \
                statistics.median(ms)
            fp64["plain_vs_pruned_max_rel"] = float(max(
                np.max(np.abs(resd[k] - res64[k]) / np.abs(res64[k]))
                for k in ('bk_raw', 'bk_shot')))
        except _lib.DeviceError as e:
            fp64["plain_full_mesh_s_per_estimate"] = None
            fp64["plain_error"] = str(e)[:200]
        finally:
            ctx.set_option('full_mesh_shells', 0)

    # B_202 diag on the same catalogue: FP32-mixed and FP64 (pruned).
    b202 = None
    if not args.no_b202:
        q32, q64 = params('fp32mixed', (2, 0, 2)), params('fp64', (2, 0, 2))
        estimate(q32, dcat)
        ms2, _, _, r2_32, _ = timed(q32, dcat, max(1, min(args.steps, 5)))
        b202 = {"s_per_estimate": round(statistics.median(ms2) / 1e3, 6)}
        if not args.no_fp64:
            estimate(q64, dcat)
            ms2d, _, _, r2_64, _ = timed(q64, dcat, 1)
            b202.update({
                "fp64_s_per_estimate": round(sum(ms2d) / 1e3, 6),
                "fp32mixed_speedup": round(sum(ms2d) /
                                           statistics.median(ms2), 2),
                "max_rel_err_fp32mixed": per_bin_err(r2_32, r2_64),
                "per_bin_detail": per_bin_err_keys(r2_32, r2_64,
                                                   ('bk_raw', 'bk_shot')),
                "nmodes_equal": bool(np.array_equal(r2_32['nmodes_1'],
                                                    r2_64['nmodes_1']))})

    variants = None
    if args.variants and fp64 is not None:
        variants = {}
        for shell64 in (0, 1):
            for shot64 in (0, 1):
                ctx.set_option('shell_fields_fp64', shell64)
                ctx.set_option('shotnoise_fp64', shot64)
                estimate(p32, dcat)
                msv, _, _, resv, _ = timed(p32, dcat, 2)
                errs = {k: [float(e) for e in
                            np.abs(resv[k] - res64[k]) / np.abs(res64[k])]
                        for k in ('bk_raw', 'bk_shot')}
                variants[f"shell64={shell64},shot64={shot64}"] = {
                    "s_per_estimate": sum(msv) / 2e3,
                    "max_rel_err": {k: max(v) for k, v in errs.items()},
                    "per_bin_rel_err": errs}
        ctx.set_option('shell_fields_fp64', 0)
        ctx.set_option('shotnoise_fp64', 0)
        ctx.set_option('sort_catalogue', 0)
        estimate(p32, dcat)
        msn, _, ktn, _, _ = timed(p32, dcat, 2, profile=True)
        variants["unsorted_catalogue"] = {
            "s_per_estimate": sum(msn) / 2e3,
            "assign_ms": round(ktn.get('assign_kernel', [0., 1])[0] / 2, 4)}
        ctx.set_option('sort_catalogue', 1)

    # Roofline of the dominant kernel of this library.
    peak, peak_kind = hbm_peak()
    mine = {k: v for k, v in ktimes.items() if not k.startswith('cufft')}
    total_k = sum(v[0] for v in ktimes.values())
    dom = max(mine, key=lambda k: mine[k][0])
    dom_ms = mine[dom][0] / mine[dom][1]
    alg = algorithmic_bytes(dom, args, 4)
    roof = None
    if alg is not None:
        ach = alg / (dom_ms * 1e-3) / 1e9
        roof = {"kernel": dom, "bound": "hbm", "achieved": round(ach, 1),
                "peak": peak, "peak_kind": f"{peak_kind} hbm_gbs",
                "unit": "GB/s", "frac": round(ach / peak, 4),
                "traffic": ncu_traffic(dom), "algorithmic_bytes": alg,
                "ms_per_launch": round(dom_ms, 4)}
        if dom.startswith('ff_'):
            roof["limiter"] = ("FP32 issue: float-float butterflies, about "
                               "100 FP32 instructions per point and stage; "
                               "the HBM fraction is not the bound")
    shares = {k: round(v[0] / total_k, 4) for k, v in
              sorted(ktimes.items(), key=lambda kv: -kv[1][0])}
    kernel_ms = total_k / nprof

    line = {
        "metric": METRIC, "value": round(value, 6), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * med_s, 3),
        "step_statistic": "median of the timed steps, max over ranks",
        "mean_ms_per_step": round(1e3 * total_s / args.steps, 3),
        "cold_first_call_s": round(cold_first_call_s, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 meshes/FFTs, f64 offsets/Ylm/reductions/shot noise",
        "data": "synthetic (seeded uniform catalogue)",
        "config": {**workload(args), "parallelism": f"replicas x{world}",
                   "evaluation_grid": list(st.get('pruned_grid', [])),
                   "autotuned": ctx.tuned()},
        "e2e": {"value": round(value_e2e, 6), "unit": UNIT,
                "h2d_bytes_per_step": int(st_e2e['h2d_bytes']),
                "d2h_bytes_per_step": int(res32['k1_bin'].size * 72)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "kernel_time_shares": shares,
        # Summed CUDA-event time of all launches of one estimate; the rest
        # of ms_per_step is host work between launches.
        "kernel_ms_per_estimate": round(kernel_ms, 3),
        "fp64": fp64,
        "b202_diag": b202,
        "precision_variants": variants,
        "clocks": clk,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"], line["oracle_check"] = cpu_baseline(
            args, norm, res32, res64)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def per_bin_err(a, b):
    """Largest per-bin relative error |a - b| / |b| (complex modulus) of
    bk_raw and bk_shot."""
    return {k: float(np.max(np.abs(a[k] - b[k]) / np.abs(b[k])))
            for k in ('bk_raw', 'bk_shot')}


def cpu_baseline(args, norm, res32, res64=None):
    """The CPU oracle on a bounded sample of the workload: the mesh set-up
    once plus two bin pairs (the lowest bin and the middle one), the
    median pair time extrapolated to the whole estimate.  The two pairs'
    normalised values are the oracle's own at the full workload size, so
    the GPU estimates are checked against them per bin."""
    from oracle.sample import GppBispecSample
    s = GppBispecSample(args.npart, args.boxsize, args.ngrid, args.nbins)
    t0 = time.perf_counter()
    s.setup()
    t_setup = time.perf_counter() - t0
    bins = [0, args.nbins // 2]
    tp, check = [], {"bins": bins, "nmodes_equal": True,
                     "rel_err_fp32mixed": {"bk_raw": [], "bk_shot": []},
                     "rel_err_fp64": {"bk_raw": [], "bk_shot": []}}
    for b in bins:
        t0 = time.perf_counter()
        s.pair(b)
        tp.append(time.perf_counter() - t0)
        raw, shot, nm = s.entry(b, norm)
        check["nmodes_equal"] &= bool(nm == res32['nmodes_1'][b])
        for name, res in (("rel_err_fp32mixed", res32), ("rel_err_fp64",
                                                         res64)):
            if res is None:
                continue
            for k, ref in (('bk_raw', raw), ('bk_shot', shot)):
                check[name][k].append(float(abs(res[k][b] - ref) / abs(ref)))
    if res64 is None:
        del check["rel_err_fp64"]
    check["max_rel_err_fp32mixed"] = max(
        max(v) for v in check["rel_err_fp32mixed"].values())
    t_pair = statistics.median(tp)
    base = {"value": round(t_setup + args.nbins * t_pair, 3), "unit": UNIT,
            "cores": s.threads, "kind": "port",
            "sample": (f"oracle set-up ({t_setup:.1f} s: assignment, "
                       f"forward FFTs, G, two-point statistics) + "
                       f"{len(bins)} of {args.nbins} bin pairs "
                       f"({t_pair:.1f} s median), extrapolated")}
    return base, check


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.sample import GppBispecSample
    s = GppBispecSample(args.npart, args.boxsize, args.ngrid, args.nbins)
    t0 = time.perf_counter()
    s.setup()
    t_setup = time.perf_counter() - t0
    for i in range(args.warmup):
        s.pair(i % args.nbins)
    tp = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        s.pair((args.warmup + i) % args.nbins)
        tp.append(time.perf_counter() - t0)
    value = t_setup + args.nbins * statistics.median(tp)
    sample = (f"oracle (numpy restatement of threept.cpp:1473-2188) set-up "
              f"{t_setup:.1f} s once + median of {args.steps} bin pairs "
              f"({statistics.median(tp):.1f} s) x {args.nbins}")
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * statistics.median(tp), 1),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded uniform catalogue)",
        "config": {**workload(args), "parallelism": "cpu"},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT,
                         "cores": s.threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 3), "unit": UNIT,
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Batched mocks: lognormal-Poisson catalogues of uneven sizes in one call.
# ---------------------------------------------------------------------------

MOCK_BOX, MOCK_NGRID = 1000., 256


def lognormal_mock(torch, dev, seed, npart, box=MOCK_BOX, n=MOCK_NGRID):
    """Poisson sample of exp(delta_G - sigma^2 / 2) - 1, delta_G Gaussian
    with P(k) = 2e4 (k / 0.02)^-1.5 exp(-(k / 0.5)^2) (Mpc/h)^3; positions
    uniform within their cell.  Returns x, y, z (float64, device)."""
    g = torch.Generator(device=dev).manual_seed(seed)
    k1 = torch.fft.fftfreq(n, d=box / n, device=dev) * 2 * np.pi
    kz = torch.fft.rfftfreq(n, d=box / n, device=dev) * 2 * np.pi
    k = torch.sqrt(k1[:, None, None] ** 2 + k1[None, :, None] ** 2 +
                   kz[None, None, :] ** 2)
    pk = 2e4 * (k.clamp_min(1e-12) / 0.02) ** -1.5 * torch.exp(-(k / 0.5) ** 2)
    pk[0, 0, 0] = 0.
    vcell = (box / n) ** 3
    white = torch.randn((n, n, n), generator=g, device=dev)
    dg = torch.fft.irfftn(torch.fft.rfftn(white) * torch.sqrt(pk / vcell),
                          s=(n, n, n))
    dln = torch.exp(dg - dg.var() / 2.) - 1.
    lam = npart * (1. + dln) / (1. + dln).sum()
    counts = torch.poisson(lam.flatten(), generator=g).to(torch.int64)
    cell = torch.repeat_interleave(torch.arange(n ** 3, device=dev), counts)
    i, j, l = cell // (n * n), (cell // n) % n, cell % n
    u = torch.rand((3, cell.numel()), generator=g, device=dev,
                   dtype=torch.float64)
    h = box / n
    return ((i + u[0]) * h, (j + u[1]) * h, (l + u[2]) * h)


def run_mocks(args):
    """Config: 256 lognormal mocks with N ~ U[2e5, 2e6], 256^3 mesh, CIC,
    B_000 and B_202 diag, 24 bins 0.005-0.245 h/Mpc, FP32-mixed, one
    batched library call per multipole."""
    import torch

    from triumvirate_gb300 import _engine, _lib
    from triumvirate_gb300.dataobjs import Binning
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(2024)
    sizes = rng.integers(200_000, 2_000_001, args.mocks)
    cols, offsets = [[], [], []], [0]
    for i, npart in enumerate(sizes):
        for c, a in zip(cols, lognormal_mock(torch, dev, 1000 + i, npart)):
            c.append(a)
        offsets.append(offsets[-1] + cols[0][-1].numel())
    x, y, z = (torch.cat(c).contiguous() for c in cols)
    del cols
    ntot = x.numel()
    counts = np.diff(offsets)
    nbar = counts / MOCK_BOX ** 3
    norms = 1. / (counts * nbar ** 2)
    binning = Binning('fourier', 'lin', 0.005, 0.245, 24)
    ctx = _lib.Context(0)
    ctx.set_option('mesh_comp', args.mesh_comp)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    cat = _engine.device_catalogue(ntot, x.data_ptr(), y.data_ptr(),
                                   z.data_ptr())

    def params(degrees, precision='fp32mixed'):
        pd = {'boxsize': {a: MOCK_BOX for a in 'xyz'},
              'ngrid': {a: MOCK_NGRID for a in 'xyz'}, 'assignment_order': 2,
              'interlace': False,
              'degrees': dict(zip(['ell1', 'ell2', 'ELL'], degrees)),
              'form': 'diag', 'shape': 'diag', 'precision': precision,
              'verbose': 0}
        return _engine.make_params(pd, '3pt')

    p000, p202 = params((0, 0, 0)), params((2, 0, 2))

    def batch():
        r0 = _engine.call_bispec_batch(ctx, p000, cat, offsets, binning,
                                       norms, shape='diag')
        r2 = _engine.call_bispec_batch(ctx, p202, cat, offsets, binning,
                                       norms, shape='diag')
        return r0, r2

    def timed_batches(steps):
        for _ in range(max(1, args.warmup)):
            batch()
        torch.cuda.synchronize(dev)
        times = []
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            batch()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            times.append(e0.elapsed_time(e1) / 1e3)
        return statistics.median(times)

    t = timed_batches(args.steps)
    graph_replays = ctx.stats()['graph_replays']

    # Accuracy against FP64 on the first mocks, and the same workload with
    # the FP32 cuFFT transforms instead of the float-float ones.
    nchk = min(4, args.mocks)
    sub = _engine.device_catalogue(int(offsets[nchk]), x.data_ptr(),
                                   y.data_ptr(), z.data_ptr())

    def max_err():
        e = {}
        for name, deg in (('B000', (0, 0, 0)), ('B202', (2, 0, 2))):
            r64 = _engine.call_bispec_batch(ctx, params(deg, 'fp64'), sub,
                                            offsets[:nchk + 1], binning,
                                            norms[:nchk], shape='diag')
            r32 = _engine.call_bispec_batch(ctx, params(deg), sub,
                                            offsets[:nchk + 1], binning,
                                            norms[:nchk], shape='diag')
            e[name] = {k: float(max(np.max(np.abs(a[k] - b[k]) / np.abs(b[k]))
                                    for a, b in zip(r32, r64)))
                       for k in ('bk_raw', 'bk_shot')}
            # The worst entry of each mock, with its modulus relative to
            # the mock's largest entry.
            e[name]['per_mock'] = [per_bin_err_keys(a, b, ('bk_raw',
                                                            'bk_shot'))
                                   for a, b in zip(r32, r64)]
            # Normwise: max |error| over max |B| of the mock.
            e[name]['normwise'] = {
                k: float(max(np.max(np.abs(a[k] - b[k])) / np.max(np.abs(b[k]))
                             for a, b in zip(r32, r64)))
                for k in ('bk_raw', 'bk_shot')}
        return e

    err_ff = max_err()
    ctx.set_option('ff_transforms', 0)
    t_fp32fft = timed_batches(max(1, min(args.steps, 2)))
    err_fp32fft = max_err()
    ctx.set_option('ff_transforms', 1)
    # Per-kernel CUDA-event time per mock of each multipole's batch call.
    per_kernel = {}
    ctx.set_option('profiling', 1)
    for name, pp in (('B000', p000), ('B202', p202)):
        _engine.call_bispec_batch(ctx, pp, cat, offsets, binning, norms,
                                  shape='diag')
        kt = ctx.kernel_times()
        per_kernel[name] = {k: round(v[0] / args.mocks, 4) for k, v in
                            sorted(kt.items(), key=lambda kv: -kv[1][0])}
    ctx.set_option('profiling', 0)
    line = {
        "metric": "batched mock bispectra (B_000 + B_202 per mock)",
        "value": round(args.mocks / t, 2), "unit": "mocks/s",
        "higher_is_better": True, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "s_per_batch": round(t, 4),
        "dtype": "f32 meshes/FFTs, f64 offsets/reductions",
        "data": "synthetic lognormal-Poisson mocks generated on the GPU",
        "config": {"workload": (f"{args.mocks} mocks, N ~ U[2e5, 2e6] "
                                f"(total {ntot}), {MOCK_NGRID}^3 mesh, CIC, "
                                "L=1000 Mpc/h, B_000 and B_202 diag, 24 lin "
                                "bins 0.005-0.245 h/Mpc"),
                   "batching": "one library call per multipole; the "
                               "largest mock warms up, the others replay "
                               "one captured CUDA graph",
                   "graph_replays_per_call": graph_replays,
                   "autotuned": ctx.tuned()},
        "kernel_ms_per_mock": per_kernel,
        "max_rel_err_vs_fp64": {"mocks": nchk, **err_ff},
        "fp32_cufft_variant": {"mocks_per_s": round(args.mocks / t_fp32fft, 2),
                               "max_rel_err_vs_fp64": err_fp32fft},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Survey bispectra: data and randoms with lines of sight (local
# plane-parallel estimator), catalogues held on the device.
# ---------------------------------------------------------------------------

def survey_catalogue(n, seed, ndata=1_000_000):
    """Observer at the origin, directions uniform on the z > 0 hemisphere,
    radii ~ N(1500, 300) Mpc/h (r > 0), nz(r) = N_data N(r; 1500, 300) /
    (2 pi r^2), FKP w_c = 1 / (1 + nz 1e4), w_s = 1."""
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(n, 3))
    u[:, 2] = np.abs(u[:, 2])
    u /= np.linalg.norm(u, axis=1)[:, None]
    r = rng.normal(1500., 300., n)
    while (r <= 0.).any():
        bad = r <= 0.
        r[bad] = rng.normal(1500., 300., int(bad.sum()))
    pdf = np.exp(-0.5 * ((r - 1500.) / 300.) ** 2) / (300. * np.sqrt(2 * np.pi))
    nz = ndata * pdf / (2 * np.pi * r ** 2)
    pos = u * r[:, None]
    return pos, nz, 1. / (1. + nz * 1e4)


def run_survey(args):
    """Config: survey bispectra from 1e6 data and 5e6 random particles
    (seeds 1, 2), 256^3 mesh, PCS (interlacing requested; three-point
    statistics turn it off), box = random extents, 20 lin bins 0.01-0.2
    h/Mpc; B_000 full (triu, 210 pairs) and B_202 full (400 pairs),
    FP32-mixed, with the Y_lm-weighted fields of all orders built in one
    fused pass and, for comparison, one order at a time; per-bin error of
    the FP32-mixed estimates against the FP64 path."""
    from triumvirate_gb300 import _lib
    from triumvirate_gb300.catalogue import DeviceCatalogue
    from triumvirate_gb300.dataobjs import Binning
    from triumvirate_gb300.threept import compute_bispec
    pd, nzd, wcd = survey_catalogue(1_000_000, 1)
    pr, nzr, wcr = survey_catalogue(5_000_000, 2)
    ctx = _lib.default_context(0)
    ctx.set_option('mesh_comp', args.mesh_comp)
    binning = Binning('fourier', 'lin', 0.01, 0.2, 20)
    samp = {'ngrid': [256] * 3, 'assignment': 'pcs', 'interlace': True,
            'precision': 'fp32mixed'}

    def cats():
        return (DeviceCatalogue(*pd.T, nz=nzd, wc=wcd),
                DeviceCatalogue(*pr.T, nz=nzr, wc=wcr))

    def estimate(degrees, form):
        dc, rc = cats()
        ctx.set_option('profiling', 0)
        t0 = time.perf_counter()
        compute_bispec(dc, rc, degrees=degrees, binning=binning, form=form,
                       sampling_params=samp)
        return time.perf_counter() - t0

    def kernel_ms(degrees, form):
        dc, rc = cats()
        ctx.set_option('profiling', 1)
        compute_bispec(dc, rc, degrees=degrees, binning=binning, form=form,
                       sampling_params=samp)
        kt = ctx.kernel_times()
        ctx.set_option('profiling', 0)
        return kt

    if args.profile_only:
        # Two B_202 estimates (for ncu captures of the survey kernels).
        for _ in range(2):
            estimate((2, 0, 2), 'full')
        return
    res = {}
    for name, degrees, form in [('B000', (0, 0, 0), 'full'),
                                ('B202', (2, 0, 2), 'full')]:
        for fused in (1, 0):
            ctx.set_option('fused_ylm', fused)
            for _ in range(max(1, args.warmup)):
                estimate(degrees, form)
            t = statistics.median(estimate(degrees, form)
                                  for _ in range(max(1, args.steps)))
            kt = kernel_ms(degrees, form)
            top = sorted(kt.items(), key=lambda kv: -kv[1][0])[:8]
            res[f"{name}.{'fused' if fused else 'per_order'}"] = {
                "s_per_estimate": round(t, 4),
                "kernel_ms": round(sum(v[0] for v in kt.values()), 2),
                "top_kernels_ms": {k: round(v[0], 3) for k, v in top}}
        ctx.set_option('fused_ylm', 1)
        if not args.no_fp64:
            dc, rc = cats()
            r32 = compute_bispec(dc, rc, degrees=degrees, binning=binning,
                                 form=form, sampling_params=samp)
            dc, rc = cats()
            r64 = compute_bispec(dc, rc, degrees=degrees, binning=binning,
                                 form=form,
                                 sampling_params={**samp, 'precision': 'fp64'})
            res[f"{name}.max_rel_err_fp32mixed_vs_fp64"] = per_bin_err_keys(
                r32, r64, ('bk_raw', 'bk_shot'))
    line = {
        "metric": "survey bispectrum s/estimate (1e6 data + 5e6 randoms, "
                  "256^3, PCS, B_202 full, 400 pairs)",
        "value": res["B202.fused"]["s_per_estimate"], "unit": "s/estimate",
        "higher_is_better": False, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 meshes/FFTs, f64 offsets/Ylm/reductions",
        "data": "synthetic (seeded hemisphere survey, FKP weights)",
        "config": {"workload": "survey B_000 full (triu) and B_202 full, "
                               "1e6 data + 5e6 randoms, 256^3, PCS, 20 lin "
                               "bins 0.01-0.2 h/Mpc, device catalogues",
                   "timing": "wall time per estimate (device-resident "
                             "catalogues, centring and lines of sight "
                             "on the device)"},
        "estimates": res,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Large mesh: a 1024^3 lognormal-Poisson box.
# ---------------------------------------------------------------------------

def per_bin_err_keys(a, b, keys):
    """Largest per-bin relative error (complex modulus) of each key, with
    the entry and its modulus relative to the largest entry."""
    out = {}
    for k in keys:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        mod = np.abs(y)
        rel = np.abs(x - y) / mod
        i = int(np.argmax(rel))
        big = mod >= 1e-3 * mod.max()
        out[k] = {"max": float(rel[i]), "entry": i,
                  "modulus_over_max": float(mod[i] / mod.max()),
                  "normwise": float(np.max(np.abs(x - y)) / mod.max()),
                  # entries not 1000x below the largest one
                  "max_above_1e-3_of_max": float(np.max(rel[big]))}
    return out


def run_large(args):
    """Config: 2e7 lognormal-Poisson particles (the mocks' P(k)) in a
    2000 Mpc/h box, 1024^3 mesh, PCS (interlacing is off for three-point
    statistics); B_000 and B_202 full form on 40 linear bins 0.005-0.3
    h/Mpc, zeta_000 and zeta_110 (diag) on 30 linear bins 10-150 Mpc/h.
    FP32-mixed timed (median of the steps), FP64 per-bin errors, per-kernel
    times and the HBM roofline of each estimate's dominant kernel."""
    import torch

    from triumvirate_gb300 import _engine, _lib
    from triumvirate_gb300.dataobjs import Binning
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(dev)
    box, ngrid, npart = 2000., 1024, 20_000_000
    x, y, z = lognormal_mock(torch, dev, 2025, npart, box=box, n=ngrid)
    torch.cuda.synchronize(dev)
    n = x.numel()
    cat = _engine.device_catalogue(n, x.data_ptr(), y.data_ptr(),
                                   z.data_ptr())
    norm = 1. / (n * (n / box ** 3) ** 2)
    ctx = _lib.Context(0)
    ctx.set_option('mesh_comp', args.mesh_comp)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    kb = Binning('fourier', 'lin', 0.005, 0.3, 40)
    rb = Binning('config', 'lin', 10., 150., 30)
    peak, peak_kind = hbm_peak()

    def params(degrees, form, precision):
        return _engine.make_params(
            {'boxsize': {a: box for a in 'xyz'},
             'ngrid': {a: ngrid for a in 'xyz'}, 'assignment_order': 4,
             'interlace': False,
             'degrees': dict(zip(['ell1', 'ell2', 'ELL'], degrees)),
             'form': form, 'shape': form, 'precision': precision,
             'verbose': 0}, '3pt')

    jobs = [('B000', 'bispec', (0, 0, 0), 'full', kb),
            ('B202', 'bispec', (2, 0, 2), 'full', kb),
            ('zeta000', '3pcf', (0, 0, 0), 'diag', rb),
            ('zeta110', '3pcf', (1, 1, 0), 'diag', rb)]
    fa = argparse.Namespace(ngrid=ngrid, npart=n, boxsize=box, nbins=40,
                            kmax=0.3)
    out = {}
    for name, kind, deg, form, binning in jobs:
        shape = 'triu' if (form == 'full' and deg[0] == deg[1]) else form
        fn = ('trvg_compute_bispec_in_gpp_box' if kind == 'bispec'
              else 'trvg_compute_3pcf_in_gpp_box')

        def est(precision):
            pp = params(deg, shape, precision)
            return _engine.call_threept(fn, ctx, pp, cat, binning, norm,
                                        kind, shape=shape)
        # Each estimate starts from a context without the cached buffers of
        # the previous ones, as a single call would (the float-float shell
        # fields of B_202 need about 104 GB).
        ctx.release_workspace()
        est('fp32mixed')
        times = []
        for _ in range(max(1, min(args.steps, 3))):
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r32 = est('fp32mixed')
            e1.record(stream)
            torch.cuda.synchronize(dev)
            times.append(e0.elapsed_time(e1) / 1e3)
        ctx.set_option('profiling', 1)
        est('fp32mixed')
        kt = ctx.kernel_times()
        ctx.set_option('profiling', 0)
        mine = {k: v for k, v in kt.items() if not k.startswith('cufft')}
        dom = max(mine, key=lambda k: mine[k][0])
        dom_ms = mine[dom][0] / mine[dom][1]
        alg = algorithmic_bytes(dom, fa, 4) if kind == 'bispec' else None
        if dom == 'reduce_pairs_tiled_kernel' and kind == 'bispec':
            # FP32 real fields on the evaluation grid: G and every field of
            # both legs (one set when the legs are equal) read once.
            mc = int(np.prod(ctx.stats()['pruned_grid']))
            nf = 40 if deg[0] == deg[1] else 80
            alg = 4 * mc * (1 + nf)
        if alg is not None and dom.startswith('ff_inv_'):
            # The table's mean counts two inverse launches (G, one leg of
            # float-float fields).  Two legs make three; and the full forms
            # reduce the fields in the tiled Gram form, which reads hi words
            # only, so the z pass writes 4 B per cell, not 8.
            g_half = algorithmic_bytes(
                dom, argparse.Namespace(**{**vars(fa), 'nbins': 0}), 4)
            ig, i_f = 2 * g_half, 2 * alg - 2 * g_half
            if dom == 'ff_inv_z_kernel':
                mc = int(np.prod(ctx.stats()['pruned_grid']))
                ig -= 4 * mc
                i_f -= 4 * mc * fa.nbins
            legs = 1 if deg[0] == deg[1] else 2
            alg = (ig + legs * i_f) / (1 + legs)
        roof = {"kernel": dom, "ms_per_launch": round(dom_ms, 4)}
        if alg is not None:
            ach = alg / (dom_ms * 1e-3) / 1e9
            roof.update({"bound": "hbm", "achieved": round(ach, 1),
                         "peak": peak, "peak_kind": f"{peak_kind} hbm_gbs",
                         "unit": "GB/s", "frac": round(ach / peak, 4),
                         "algorithmic_bytes": alg})
        entry = {"s_per_estimate": round(statistics.median(times), 4),
                 "entries": int(np.asarray(r32['k1_bin' if kind == 'bispec'
                                               else 'r1_bin']).size),
                 "kernel_ms": round(sum(v[0] for v in kt.values()), 2),
                 "top_kernels_ms": {k: round(v[0], 3) for k, v in sorted(
                     kt.items(), key=lambda kv: -kv[1][0])[:6]},
                 "roofline_dominant": roof,
                 "evaluation_grid": list(ctx.stats()['pruned_grid']),
                 "shell_transforms": ("float-float" if any(
                     k.startswith('ff_') for k in kt) else "FP32 cuFFT")}
        if not args.no_fp64:
            t0 = time.perf_counter()
            r64 = est('fp64')
            torch.cuda.synchronize(dev)
            entry["fp64_s_per_estimate"] = round(time.perf_counter() - t0, 3)
            keys = (('bk_raw', 'bk_shot') if kind == 'bispec'
                    else ('zeta_raw', 'zeta_shot'))
            entry["max_rel_err_fp32mixed"] = per_bin_err_keys(r32, r64, keys)
            cnt = 'nmodes_1' if kind == 'bispec' else 'npairs_1'
            entry["counts_equal"] = bool(np.array_equal(r32[cnt], r64[cnt]))
            if kind == 'bispec':
                # The same estimate with FP32 cuFFT shell fields (option
                # ff_transforms = 0) instead of the float-float transforms.
                ctx.set_option('ff_transforms', 0)
                try:
                    est('fp32mixed')
                    t32 = []
                    for _ in range(2):
                        torch.cuda.synchronize(dev)
                        e0 = torch.cuda.Event(enable_timing=True)
                        e1 = torch.cuda.Event(enable_timing=True)
                        e0.record(stream)
                        rf = est('fp32mixed')
                        e1.record(stream)
                        torch.cuda.synchronize(dev)
                        t32.append(e0.elapsed_time(e1) / 1e3)
                finally:
                    ctx.set_option('ff_transforms', 1)
                entry["fp32_fft_variant"] = {
                    "s_per_estimate": round(statistics.median(t32), 4),
                    "max_rel_err_vs_fp64": per_bin_err_keys(rf, r64, keys)}
        out[name] = entry
        print(f"# {name}: {json.dumps(entry)}", file=sys.stderr, flush=True)
    line = {
        "metric": "large-mesh estimates s/estimate (1024^3, 2e7 lognormal "
                  "particles, PCS)",
        "value": out['B000']['s_per_estimate'], "unit": "s/estimate",
        "higher_is_better": False, "n_gpus": 1, "steps": args.steps,
        "warmup": 1, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 meshes / float-float transforms, f64 "
                 "offsets/reductions",
        "data": "synthetic lognormal-Poisson box generated on the GPU",
        "config": {"workload": (f"{n} lognormal-Poisson particles, L=2000 "
                                "Mpc/h, 1024^3 mesh, PCS; B_000 and B_202 "
                                "full 40 lin bins 0.005-0.3 h/Mpc; zeta_000 "
                                "and zeta_110 diag 30 lin bins 10-150 "
                                "Mpc/h")},
        "estimates": out,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == 'reference':
        run_reference(args)
    elif args.workload == 'mocks':
        run_mocks(args)
    elif args.workload == 'survey':
        run_survey(args)
    elif args.workload == 'large':
        run_large(args)
    else:
        run_gb300(args)


if __name__ == '__main__':
    main()
