"""Benchmark: polychromatic 1024^2 PSFs/s of the broadband segmented workload.

Workload (one "step" = 32 PSFs through the fused broadband plan, each with
its own OPD map): 1024x1024 pupil of 18 hexagonal segments (two rings, empty
centre, 2 px gaps), per-segment piston/tip/tilt ~ N(0, 50 nm), global Noll
2-22 ~ N(0, 15 nm), 64 wavelengths over 500-900 nm weighted by a 5800 K
blackbody, 512x512 detector at oversample 2 (1024^2 field per wavelength).
Inputs are seeded synthetic arrays of those shapes.  The timed region runs a
step's PSFs over two streams (PSFPlan.execute_streams); per-kernel times for
the rooflines come from the same steps run serially right after it.

Arms:
  default           the split-precision tensor-core plan (lentil_gb300) on cuda
  --impl reference  lentil 0.8.8 itself (installed under baseline/_ref; else
                    the numpy restatement under oracle/) on the host cores,
                    a bounded sample of wavelengths per step

Prints ONE JSON line (rank 0).  Under torchrun every rank runs an independent
replica on its own GPU (the path has no data exchange); value is the total
PSFs of all ranks over the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'polychromatic 1024^2 PSFs/s (broadband segmented, 64 wavelengths), split precision'
UNIT = 'PSFs/s'
PEAKS_FILE = os.path.join(ROOT, 'MEASURED_PEAKS.json')
TRAFFIC_FILE = os.path.join(ROOT, 'profiles', 'mft_split_broadband_segmented.json')


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=30)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--psfs-per-step', type=int, default=32,
                    help='PSFs per step (each with its own OPD map), one plan execute each')
    ap.add_argument('--precision', default='split-bf16',
                    choices=['split-fp16', 'split-bf16', 'fp64'])
    ap.add_argument('--fp64-steps', type=int, default=2,
                    help='timed steps of the plain complex128 plan (0 to skip)')
    ap.add_argument('--cpu-lambdas', type=int, default=4,
                    help='wavelengths in the bounded CPU-baseline sample (reference arm: per step)')
    ap.add_argument('--npix', type=int, default=1024)
    ap.add_argument('--wavelengths', type=int, default=64)
    ap.add_argument('--rates', default='10,50,200,500,1000,2000',
                    help='serving: Poisson arrival rates (requests/s)')
    ap.add_argument('--duration', type=float, default=4.0, help='serving: seconds per rate')
    ap.add_argument('--max-requests', type=int, default=1000,
                    help='serving: at most this many requests per rate')
    ap.add_argument('--serve-warm', type=float, default=4.0,
                    help='serving: seconds of the warm pass at 100 requests/s')
    ap.add_argument('--serve-streams', type=int, default=4,
                    help='serving: CUDA streams of the server (launches in flight)')
    ap.add_argument('--serve-batch', type=int, default=8,
                    help='serving: requests batched into one launch at most')
    ap.add_argument('--serving-leg', type=int, default=1,
                    help='default workload: 1 = add a short serving leg (p50/p99) to the line')
    ap.add_argument('--serving-leg-rates', default='200,1000',
                    help='default workload: Poisson rates of the serving leg')
    ap.add_argument('--tile', type=int, default=0, choices=[0, 128, 256],
                    help='tensor-core MFT pair-tile width: 0 = the autotuner\'s choice '
                         '(measured per launch shape), 128 or 256 = forced')
    ap.add_argument('--tune', default='measure', choices=['measure', 'model'],
                    help='autotuner mode when --tile is 0: time both widths online per '
                         'launch class, or take the occupancy model\'s choice')
    ap.add_argument('--workload', default='broadband',
                    choices=['broadband', 'monochromatic', 'phase_retrieval', 'serving', 'large'],
                    help='broadband: the headline workload; the others measure the '
                         'monochromatic 256^2 PSF and the focus-diverse gradient')
    return ap.parse_args()


def config_dict(wl, args, extra=None):
    d = {'workload': 'broadband segmented PSF: 1024^2 pupil, 18 hex segments (2 rings, '
                     'empty centre, 2 px gaps), per-segment PTT N(0,50nm), Noll 2-22 '
                     'N(0,15nm), 64 wavelengths 500-900 nm, 5800 K blackbody, 512^2 '
                     'detector x oversample 2',
         'pupil': list(wl.plane_shape), 'wavelengths': len(wl.wavelengths),
         'output': [wl.det_shape * wl.oversample] * 2, 'psfs_per_step': getattr(args, 'psfs_per_step', 1),
         'optics': 'D = 1 m over the pupil grid, f = 10 m, 5 um pixels',
         'l2': 'working set (DFT matrices + per-wavelength operands, > 1 GB) exceeds the '
               '129 MB L2; no flush needed'}
    if extra:
        d.update(extra)
    return d


# --------------------------------------------------------------------------
# CPU reference: lentil itself (when installed beside the repository) or its
# algorithm restated in numpy (oracle/), on the host cores
# --------------------------------------------------------------------------
LENTIL_DIR = os.path.join(ROOT, 'baseline', '_ref')


def reference_module():
    """(module, kind, label): lentil 0.8.8 from ``baseline/_ref`` when it is
    installed there, else the numpy restatement under ``oracle/``.  Both
    expose lentil's Pupil / Wavefront / propagate_dft / insert."""
    if os.path.isfile(os.path.join(LENTIL_DIR, 'lentil', '__init__.py')):
        if LENTIL_DIR not in sys.path:
            sys.path.append(LENTIL_DIR)
        try:
            import lentil
            return lentil, 'reference', f'lentil {lentil.__version__} stock numpy path'
        except Exception:            # an unusable install: fall back to the port
            pass
    from oracle import lentil_oracle as lo
    return lo, 'port', 'numpy restatement of lentil (oracle/)'


def cpu_reference(wl, idx, opd):
    """lentil's documented user loop over the wavelengths ``idx`` of one PSF:
    Wavefront(lam) * pupil -> propagate_dft -> insert(img, weight)
    (docs/user/performance.rst:44-49), one field per segment mask.
    Returns (seconds, image, kind, label)."""
    mod, kind, label = reference_module()
    pupil = mod.Pupil(amplitude=wl.amp, opd=opd, mask=wl.mask3d, pixelscale=wl.pixelscale_in,
                      focal_length=wl.focal_length)
    img = None
    t0 = time.perf_counter()
    for lam, w in zip(wl.wavelengths[idx], wl.weights[idx]):
        wf = mod.propagate_dft(mod.Wavefront(lam) * pupil, wl.det_pixelscale, shape=wl.det_shape,
                               oversample=wl.oversample)
        img = wf.insert(np.zeros(wf.shape) if img is None else img, weight=w)
    return time.perf_counter() - t0, img, kind, label


def sample_indices(L, n, k=0):
    """``n`` wavelength indices spread over ``L``, rotated by step ``k``."""
    return (np.arange(n) * max(1, L // n) + k) % L


def run_reference(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    from lentil_gb300 import workloads
    from oracle import lentil_oracle as lo
    # the same seeded workload, its Zernike modes evaluated on the host
    wl = workloads.broadband_segmented(args.npix, args.wavelengths, basis=lo.zernike_basis)
    opd = wl.opds(1)[0]
    L = len(wl.wavelengths)
    # each step is a bounded sample of one PSF: --cpu-lambdas of its L
    # wavelengths (rotating through the band from step to step)
    n = min(L, max(1, args.cpu_lambdas))
    for k in range(max(1, min(args.warmup, 2))):
        cpu_reference(wl, sample_indices(L, 1, k), opd)
    per = []
    for k in range(args.steps):
        dt, _, kind, label = cpu_reference(wl, sample_indices(L, n, k), opd)
        per.append(dt)
    step_s = statistics.mean(per)
    value = (n / L) / step_s                       # PSFs per second (fractions of one PSF)
    cores = os.cpu_count()
    sample = (f'{n} of {L} wavelengths of one PSF per step through lentil\'s per-segment user '
              f'loop ({label}); value = PSF fraction per step / measured step time')
    line = {'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT,
            'n_gpus': args.gpus, 'device': 'host CPU cores (the arm uses no GPU)',
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * step_s,
            'psf_fraction_per_step': n / L,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic', 'config': config_dict(wl, args),
            'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': cores, 'kind': kind,
                             'sample': sample},
            'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks/throttle sampling while the timed region runs.

    The sampler is started first and the timed region begins only once it has
    produced a sample (nvidia-smi takes ~1 s to start); samples are stamped on
    arrival and only those inside the timed region are summarised."""
    Q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index, self.proc, self.stamped = index, None, []
        self.t_in = self.t_out = None

    def _reader(self):
        for ln in self.proc.stdout:
            if ln.strip():
                self.stamped.append((time.perf_counter(), ln))

    def __enter__(self):
        import threading
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), f'--query-gpu={self.Q}',
                 '--format=csv,noheader,nounits', '-lms', '50'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self
        threading.Thread(target=self._reader, daemon=True).start()
        t0 = time.perf_counter()
        while not self.stamped and time.perf_counter() - t0 < 5.0:
            time.sleep(0.02)
        self.t_in = time.perf_counter()
        return self

    def __exit__(self, *exc):
        self.t_out = time.perf_counter()
        if self.proc is not None:
            time.sleep(0.06)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.proc.wait()

    def summary(self):
        sm, smax, power, reasons = [], [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        lines = [ln for t, ln in self.stamped
                 if self.t_in is not None and self.t_in <= t <= self.t_out]
        for ln in lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0])); smax.append(float(f[1])); power.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower() == 'active':
                    reasons.add(name)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': [], 'samples': 0}
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(smax),
                'power_w_max': max(power), 'reasons': sorted(reasons), 'samples': len(sm),
                'window_s': self.t_out - self.t_in}


def slowest_rank(ms_local, units_per_rank, world, device):
    """Whole-job throughput of independent replicas: the slowest rank's time
    (MAX over ranks) and the units all ranks processed in it.  The path has
    no data exchange; the one collective is this reduction of the clock."""
    ms = float(ms_local)
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * units_per_rank / (ms / 1e3)


def peaks():
    try:
        with open(PEAKS_FILE) as fh:
            d = json.load(fh)
        return d, 'measured'
    except (OSError, ValueError):
        return {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0, 'bf16_tflops_sustained': 1700.0}, 'fallback'


def traffic_per_launch():
    try:
        with open(TRAFFIC_FILE) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return None


def fp64_gemm_peaks(dev, n=2048, reps=5):
    """Measured FP64 rates of this GPU in the same run: cuBLAS complex128 and
    float64 GEMMs (torch.matmul) of n x n x n, best of ``reps``; TFLOP/s
    counting 8 n^3 (complex) and 2 n^3 (real) flops."""
    import torch
    out = {}
    for name, dt, fl in (('zgemm', torch.complex128, 8.0), ('dgemm', torch.float64, 2.0)):
        a = torch.randn(n, n, dtype=dt, device=dev)
        b = torch.randn(n, n, dtype=dt, device=dev)
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name + '_tflops'] = fl * n ** 3 / (best / 1e3) / 1e12
        del a, b
    out['how'] = f'torch.matmul {n}^3, best of {reps}, CUDA events'
    return out


def run_gpu(args):
    import torch
    import torch.distributed as dist
    import lentil_gb300 as lg
    from lentil_gb300 import _lib, broadband, workloads

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group('nccl', device_id=torch.device('cuda', local))

    def barrier():
        if world > 1:
            dist.barrier()

    wl = workloads.broadband_segmented(args.npix, args.wavelengths)
    P = args.psfs_per_step
    gmask = wl.mask3d.sum(axis=0)
    amp_eff = wl.amp * gmask                       # lentil: amplitude[s] * mask[s]
    opd = wl.opds(P, seed=wl.seed + rank)          # a distinct OPD map per PSF of a step
    s = lg.util.boundary_slice(gmask)
    geo = broadband.plan_geometry(wl.plane_shape, s, [], np.broadcast_to(wl.pixelscale_in, (2,)),
                                  wl.focal_length, lg.pupil, wl.wavelengths, wl.det_pixelscale,
                                  shape=wl.det_shape, oversample=wl.oversample)
    L = len(geo.wavelengths)
    dev = torch.device('cuda', local)
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    plan = broadband.make_plan(geo, batch=1, precision=args.precision)
    torch.cuda.synchronize()
    plan_ms = 1e3 * (time.perf_counter() - t0)

    A = torch.as_tensor(amp_eff[None], device=dev)
    O = torch.as_tensor(opd, device=dev)           # [P, H, W]
    Wt = torch.as_tensor(wl.weights[geo.keep][None], device=dev)
    out = torch.empty((P,) + geo.shape_out, dtype=torch.float64, device=dev)
    lib = _lib.load()

    def step(a, o, w, img):
        # the step's PSFs alternate over two streams with a workspace each
        # (PSFPlan.execute_streams), joined back to the current stream
        plan.execute_streams(a, o, w, img, check=False)

    def step_serial(a, o, w, img):
        # the same PSFs one after the other on the current stream
        for k in range(P):
            plan.execute(a, o[k:k + 1], w, out=img[k:k + 1], check=False)

    # ---------------- device-resident timed region (value) ----------------
    for _ in range(args.warmup):
        step(A, O, Wt, out)
    _lib.call('lgb_psf_plan_status', plan._h, stream.cuda_stream)
    plan.stream_status()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for k in range(args.steps):
            ev[k][0].record(stream)
            step(A, O, Wt, out)
            ev[k][1].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize()
    barrier()
    plan.stream_status()
    step_ms = sorted(a.elapsed_time(b) for a, b in ev)

    # ---------------- kernel-timing region (roofline) ----------------------
    # Per-kernel CUDA-event times need serialised launches: in the timed
    # region the two lanes overlap one PSF's kernels with the next one's, so
    # an event pair there would also count the wait for the other lane's
    # CTA pairs.  The same steps again, one PSF after the other on the
    # current stream, with the plan's profiler on.
    import ctypes
    for _ in range(2):
        step_serial(A, O, Wt, out)
    lib.lgb_psf_plan_profile(plan._h, 1)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as kclk:
        k_start = torch.cuda.Event(enable_timing=True)
        k_end = torch.cuda.Event(enable_timing=True)
        k_start.record(stream)
        for _ in range(args.steps):
            step_serial(A, O, Wt, out)
        k_end.record(stream)
        torch.cuda.synchronize()
    barrier()
    lib.lgb_psf_plan_profile(plan._h, 0)
    kernel_region_ms = k_start.elapsed_time(k_end)
    kms = (ctypes.c_double * 4)()
    kcnt = (ctypes.c_int * 4)()
    _lib.call('lgb_psf_plan_kernel_times', plan._h, kms, kcnt, 4)
    _lib.call('lgb_psf_plan_status', plan._h, stream.cuda_stream)
    region_ms = t_start.elapsed_time(t_end)
    total_ms, value = slowest_rank(region_ms, P * args.steps, world, dev)

    # ---------------- end-to-end through the plan with host buffers --------
    # Every step copies its PSFs' amp/opd/weights from pinned host memory and
    # reads their images back; a copy stream moves step k+1's inputs and step
    # k's images while the compute stream runs, with double-buffered device
    # buffers and events ordering every reuse.
    hA = A.cpu().pin_memory()
    hO = O.cpu().pin_memory()
    hW = Wt.cpu().pin_memory()
    hOut = [torch.empty_like(out, device='cpu').pin_memory() for _ in range(2)]
    dA = [torch.empty_like(A) for _ in range(2)]
    dO = [torch.empty_like(O) for _ in range(2)]
    dW = [torch.empty_like(Wt) for _ in range(2)]
    dOut = [torch.empty_like(out) for _ in range(2)]
    copy = torch.cuda.Stream(device=dev)

    def load_inputs(b):                              # the step's pupil amplitude and weights,
        dA[b].copy_(hA, non_blocking=True)           # and one OPD map per PSF
        dO[b].copy_(hO, non_blocking=True)
        dW[b].copy_(hW, non_blocking=True)

    def e2e_run(n):
        ready = [torch.cuda.Event() for _ in range(2)]
        done = [torch.cuda.Event() for _ in range(2)]
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(copy)
        with torch.cuda.stream(copy):
            load_inputs(0)
        ready[0].record(copy)
        for k in range(n):
            b = k & 1
            stream.wait_event(ready[b])
            step(dA[b], dO[b], dW[b], dOut[b])
            done[b].record(stream)
            with torch.cuda.stream(copy):
                if k + 1 < n:
                    nb = 1 - b
                    if k >= 1:
                        copy.wait_event(done[nb])       # step k-1 no longer reads buffer nb
                    load_inputs(nb)
                    ready[nb].record(copy)
                copy.wait_event(done[b])
                hOut[b].copy_(dOut[b], non_blocking=True)
        t1.record(copy)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1)

    e2e_run(max(2, args.warmup))
    barrier()
    torch.cuda.synchronize()
    e2e_ms = e2e_run(args.steps)
    barrier()
    plan.stream_status()
    if not torch.equal(hOut[(args.steps - 1) & 1], dOut[(args.steps - 1) & 1].cpu()):
        raise RuntimeError('end-to-end image read back differs from the device image')
    e2e_ms, e2e_value = slowest_rank(e2e_ms, P * args.steps, world, dev)
    h2d = (A.numel() + O.numel() + Wt.numel()) * 8
    d2h = out.numel() * 8

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # ---------------- accuracy vs the plain complex128 plan ----------------
    split_img = torch.empty_like(out[:1])
    plan.execute(A, O[:1], Wt, out=split_img)
    fp64_value = fp64_err = None
    fp64_ms = None
    fp64_peaks = None
    if args.fp64_steps > 0 and args.precision != 'fp64':
        plan64 = broadband.make_plan(geo, batch=1, precision='fp64')
        ref = torch.empty_like(split_img)
        plan64.execute(A, O[:1], Wt, out=ref)      # warm-up and reference
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.fp64_steps):
            plan64.execute(A, O[:1], Wt, out=ref, check=False)
        f1.record(stream)
        torch.cuda.synchronize()
        fp64_ms = f0.elapsed_time(f1) / args.fp64_steps
        fp64_value = 1.0 / (fp64_ms / 1e3)
        fp64_err = float(((split_img - ref).abs().amax() / ref.abs().amax()).item())
        del plan64, ref
        fp64_peaks = fp64_gemm_peaks(dev)

    # ---------------- roofline of the dominant kernel ----------------------
    m, n = geo.fslice[2], geo.fslice[3]
    M, N = geo.window_shape
    flops_stage1 = 8.0 * M * m * n * L            # complex MACs x 8 (algorithmic), per PSF
    flops_stage2 = 8.0 * M * n * N * L
    mft_ms = kms[1] + kms[2]
    launches = kcnt[1] + kcnt[2]
    psfs = P * args.steps
    pk, pk_kind = peaks()
    # the burst figure for a timed region under a second (the clock has not
    # settled under the power limit yet), the sustained one for longer runs
    sustained = kernel_region_ms >= 1000.0
    peak = pk.get('bf16_tflops_sustained' if sustained else 'bf16_tflops', pk.get('bf16_tflops'))
    achieved = (flops_stage1 + flops_stage2) * psfs / (mft_ms / 1e3) / 1e12
    # stage 1 issues only the K blocks whose field rows are nonzero somewhere
    # in the column tile (the tile width of the timed launches)
    r0, c0 = geo.fslice[0], geo.fslice[1]
    width = lg.tuner.last_tile() or 256
    live = stage1_live_fraction(amp_eff[r0:r0 + m, c0:c0 + n] != 0, width) \
        if args.precision != 'fp64' else 1.0
    issued = 3 * (flops_stage1 * live + flops_stage2) * psfs / (mft_ms / 1e3) / 1e12
    tr = traffic_per_launch()
    roofline = {'bound': 'tensor', 'kernel': 'split_mft_kernel (tcgen05, both MFT stages)',
                'achieved': achieved, 'peak': peak, 'unit': 'TFLOP/s', 'frac': achieved / peak,
                'peak_kind': f'{pk_kind} bf16 dense, ' + ('sustained (timed region >= 1 s)'
                                                          if sustained else
                                                          'burst (timed region < 1 s)'),
                'timed_region_ms': kernel_region_ms,
                'region_note': 'kernel times from a profiled region of the same steps run '
                               'serially (one PSF after the other on one stream) right after '
                               'the timed region, whose two lanes overlap the kernels of '
                               'consecutive PSFs',
                'serial_psfs_per_s': psfs / (kernel_region_ms / 1e3),
                # the timed (two-lane) region itself: algorithmic MFT flops
                # over its wall time, a lower bound on the kernels' rate (the
                # step also runs the phasor operand and window kernels)
                'timed_region_tflops_lower_bound':
                    (flops_stage1 + flops_stage2) * psfs / (region_ms / 1e3) / 1e12,
                'timed_region_frac_lower_bound':
                    (flops_stage1 + flops_stage2) * psfs / (region_ms / 1e3) / 1e12 / peak,
                'clocks': kclk.summary(),
                'issued_tflops': issued,
                'issued_note': 'three split products per algorithmic flop; stage 1 counts '
                               'its issued K blocks only (stage1_live_fraction); padding '
                               'not counted',
                'stage1_live_fraction': live,
                'traffic': tr.get('traffic_bytes_per_launch') if tr else None,
                'traffic_note': tr.get('note') if tr else 'no ncu capture committed',
                'launches': launches, 'avg_launch_ms': mft_ms / max(1, launches),
                'algorithmic_flops_per_psf': flops_stage1 + flops_stage2,
                'kernel_ms_per_psf': {name: kms[i] / psfs
                                      for i, name in enumerate(_lib.PROFILE_SLOTS)}}

    # ---------------- HBM rooflines of the elementwise kernels ---------------
    # algorithmic bytes per launch: the phasor writes the split stage-1
    # operand (hi + lo planes of f^T, n x 2 kp1 x 2 B each, per wavelength)
    # after reading amp and opd over the field slice; the window add reads the
    # FP32 window and read-modify-writes the float64 image
    kp1 = (m + 31) // 32 * 32
    hbm = pk.get('hbm_gbs', 6800.0)

    def hbm_roofline(ms, nbytes, note=None):
        gbs = nbytes / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        r = {'ms_per_launch': ms, 'algorithmic_bytes': nbytes, 'achieved_gbs': gbs,
             'peak_gbs': hbm, 'frac': gbs / hbm, 'peak_kind': f'{pk_kind} HBM copy'}
        if note:
            r['note'] = note
        return r

    elementwise = {
        'split_field_T_kernel': hbm_roofline(kms[0] / max(1, kcnt[0]),
                                             L * n * 2 * kp1 * 2 * 2 + 16 * m * n),
        'window_add_kernel': hbm_roofline(kms[3] / max(1, kcnt[3]), M * N * (4 + 16),
                                          'a 1024^2 window (20 MB) stays in the 129 MB L2'),
    }

    # ---------------- the drop-in API with host arrays ----------------------
    # lentil-style call: numpy pupil (amplitude, OPD, 18 segment masks) in,
    # numpy image out; host preparation, copies and the plan execute included
    pup = lg.Pupil(amplitude=wl.amp, opd=opd[0], mask=wl.mask3d, pixelscale=wl.pixelscale_in,
                   focal_length=wl.focal_length)
    api = lambda: lg.broadband_psf(pup, wl.wavelengths, wl.weights, wl.det_pixelscale,
                                   shape=wl.det_shape, oversample=wl.oversample,
                                   precision=args.precision)
    api()
    torch.cuda.synchronize()
    a0 = time.perf_counter()
    for _ in range(3):
        api()
    api_s = (time.perf_counter() - a0) / 3
    pup.freeze()                                   # lentil's Plane.freeze: amp/opd fixed
    api()
    a0 = time.perf_counter()
    for _ in range(5):
        api()
    api_frozen_s = (time.perf_counter() - a0) / 5

    # ---------------- CPU baseline and error vs the reference ---------------
    # a bounded sample: --cpu-lambdas wavelengths of PSF 0 through lentil's
    # per-segment loop on the host, and the same wavelengths through the plan
    n_cpu = min(L, max(1, args.cpu_lambdas))
    idx = sample_indices(L, n_cpu)
    cpu_s, cpu_img, cpu_kind, cpu_label = cpu_reference(wl, idx, opd[0])
    cpu_value = (n_cpu / L) / cpu_s
    sub = torch.as_tensor(idx.astype(np.int32), device=dev)
    sub_img = plan.execute(A, O[:1], torch.as_tensor(wl.weights[idx][None], device=dev),
                           lam_idx=sub)[0].cpu().numpy()
    err_ref = float(np.abs(sub_img - cpu_img).max() / np.abs(cpu_img).max())

    # ---------------- plan build once memory is cached ----------------------
    # the first build above mapped new device memory for the plan; a plan
    # built after another of the same size was released reuses that block
    del plan
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan = broadband.make_plan(geo, batch=1, precision=args.precision)
    torch.cuda.synchronize()
    rebuild_ms = 1e3 * (time.perf_counter() - t0)

    serving_leg = run_serving_leg(args) if args.serving_leg else None

    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': total_ms / args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None,
        'dtype': {'split-fp16': 'fp16 hi+lo split operands, fp32 accumulate',
                  'split-bf16': 'bf16 hi+lo split operands, fp32 accumulate',
                  'fp64': 'f64 (complex128)'}[args.precision],
        'data': 'synthetic (seeded)',
        'config': config_dict(wl, args, {'precision': args.precision,
                                         'field': [m, n], 'window': [M, N],
                                         'parallelism': f'replicas x{world}',
                                         'mft_tile': tuner_summary(args)}),
        'psfs_per_step': P,
        'p50_ms': statistics.median(step_ms), 'p99_ms': float(np.percentile(step_ms, 99)),
        'plan_build_ms': plan_ms,
        'plan_rebuild_ms': rebuild_ms,
        'plan_note': 'plan_build_ms: the first plan of the process (its device memory newly '
                     'mapped); plan_rebuild_ms: the same plan built again after the first was '
                     'released (memory from the caching allocator): DFT matrices of all '
                     'wavelengths plus host set-up',
        'err_vs_fp64': fp64_err,
        'err_vs_oracle': {'value': err_ref, 'wavelengths': idx.tolist(), 'oracle': cpu_label,
                          'note': 'peak-normalised, the plan on these wavelengths vs the '
                                  'host loop on the same inputs'},
        'fp64_plain': None if fp64_value is None else {
            'value': fp64_value, 'unit': UNIT, 'ms_per_psf': fp64_ms,
            'speedup_split_over_fp64': value / world / fp64_value,
            'roofline': {'bound': 'fp64', 'achieved': (flops_stage1 + flops_stage2) / (fp64_ms / 1e3) / 1e12,
                         'peak': fp64_peaks['zgemm_tflops'], 'unit': 'TFLOP/s',
                         'frac': (flops_stage1 + flops_stage2) / (fp64_ms / 1e3) / 1e12
                                 / fp64_peaks['zgemm_tflops'],
                         'peak_kind': 'cuBLAS complex128 GEMM measured in this run',
                         'measured_fp64_peaks': fp64_peaks,
                         'note': 'whole plan execute (phasor, both GEMMs, intensity) against '
                                 'the algorithmic MFT flops'}},
        'roofline': roofline,
        'elementwise_roofline': elementwise,
        'dropin_api': {'value': 1.0 / api_s, 'unit': UNIT,
                       'frozen_pupil': 1.0 / api_frozen_s,
                       'path': 'lentil_gb300.broadband_psf(Pupil of numpy amplitude, OPD and 18 '
                               'segment masks) -> numpy image (host preparation, copies, '
                               'cached plan execute, read-back); frozen_pupil: the same after '
                               'Pupil.freeze(), whose merged field stays on the device'},
        'cpu_baseline': {'value': cpu_value, 'unit': UNIT, 'cores': os.cpu_count(),
                         'kind': cpu_kind,
                         'sample': f'{n_cpu} of {L} wavelengths of one PSF through lentil\'s '
                                   f'per-segment user loop ({cpu_label}); value = PSF fraction '
                                   '/ measured time'},
        'e2e': {'value': e2e_value, 'unit': UNIT, 'h2d_bytes_per_step': h2d,
                'd2h_bytes_per_step': d2h,
                'path': 'PSFPlan.execute_streams on pinned-host amp/opd/weights copied in and '
                        'the images copied out every step; copies on a third stream overlap '
                        'the previous/next step\'s compute'},
        # the library's kernels in the timed region: the plan profiler's
        # launch counts (phasor operand, both MFT stages, window add) over the
        # serial profiled region, which issues the same launches for the same
        # steps, plus the per-PSF max reduction that only the fp16 form runs
        'gpu_launches': int(sum(kcnt[i] for i in range(4))) +
                        (P * args.steps if args.precision == 'split-fp16' else 0),
        'clocks': clk.summary(),
    }
    if serving_leg:
        line['serving'] = serving_leg
        line['serving_p50_ms'] = serving_leg['rates'][0]['p50_ms']
        line['serving_p99_ms'] = serving_leg['rates'][0]['p99_ms']
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def _timed(fn, steps, warmup):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    s = torch.cuda.current_stream()
    for a, b in ev:
        a.record(s)
        fn()
        b.record(s)
    torch.cuda.synchronize()
    ms = sorted(a.elapsed_time(b) for a, b in ev)
    return statistics.mean(ms), statistics.median(ms), float(np.percentile(ms, 99))


def run_monochromatic(args):
    """256^2 circular pupil, Noll 2-11, 650 nm, 128^2 detector x2: lentil's
    propagate_dft + intensity through the drop-in API (complex128) and the
    fused plan (split), against the oracle."""
    import torch
    import lentil_gb300 as lg
    from lentil_gb300 import broadband, workloads
    from oracle import lentil_oracle as lo
    wl = workloads.monochromatic_circle()
    opd = wl.opds(1)[0]
    pl = lg.Pupil(amplitude=wl.amp, opd=opd, pixelscale=wl.pixelscale_in, focal_length=wl.focal_length)
    api = lambda: lg.propagate_dft(lg.Wavefront(650e-9) * pl, wl.det_pixelscale, shape=wl.det_shape,
                                   oversample=wl.oversample).intensity_tensor()
    api_mean, api_p50, api_p99 = _timed(api, args.steps, args.warmup)
    s = lg.util.boundary_slice(wl.amp)
    geo = broadband.plan_geometry(wl.plane_shape, s, [], np.broadcast_to(wl.pixelscale_in, (2,)),
                                  wl.focal_length, lg.pupil, wl.wavelengths, wl.det_pixelscale,
                                  shape=wl.det_shape, oversample=wl.oversample)
    plan = broadband.make_plan(geo, batch=1, precision=args.precision)
    A = torch.as_tensor(wl.amp[None], device='cuda')
    O = torch.as_tensor(opd[None], device='cuda')
    W = torch.ones((1, 1), dtype=torch.float64, device='cuda')
    out = torch.empty((1,) + geo.shape_out, dtype=torch.float64, device='cuda')
    fused = lambda: plan.execute(A, O, W, out=out, check=False)
    e_mean, e_p50, e_p99 = _timed(fused, args.steps, args.warmup)
    fused_tile = tuner_summary(args)
    cap = plan.capture(A, O, W, out)                # the same execute as one CUDA graph
    f_mean, f_p50, f_p99 = _timed(cap.replay, args.steps, args.warmup)
    cap.status()
    ref_pl = lo.Pupil(amplitude=wl.amp, opd=opd, pixelscale=wl.pixelscale_in, focal_length=wl.focal_length)
    ref = lo.propagate_dft(lo.Wavefront(650e-9) * ref_pl, wl.det_pixelscale, shape=wl.det_shape,
                           oversample=wl.oversample).intensity
    # CPU baseline: lentil itself where installed (else the oracle port)
    mod, kind, label = reference_module()
    cpu_pl = mod.Pupil(amplitude=wl.amp, opd=opd, pixelscale=wl.pixelscale_in,
                       focal_length=wl.focal_length)
    t0 = time.perf_counter()
    for _ in range(5):
        mod.propagate_dft(mod.Wavefront(650e-9) * cpu_pl, wl.det_pixelscale, shape=wl.det_shape,
                          oversample=wl.oversample).intensity
    cpu_s = (time.perf_counter() - t0) / 5
    e_api = lo.peak_normalised_error(api().cpu().numpy(), ref)
    e_fused = lo.peak_normalised_error(plan.execute(A, O, W).cpu().numpy()[0], ref)
    # propagate_fft on the same pupil (666^2 centred FFT, cropped to 256^2):
    # the drop-in API in complex128 and split precision vs numpy's FFT
    fft_legs = {}
    ref_fft = lo.propagate_fft(lo.Wavefront(650e-9) * ref_pl, wl.det_pixelscale, shape=wl.det_shape,
                               oversample=wl.oversample).intensity
    t0 = time.perf_counter()
    mod.propagate_fft(mod.Wavefront(650e-9) * cpu_pl, wl.det_pixelscale, shape=wl.det_shape,
                      oversample=wl.oversample).intensity
    cpu_fft_s = time.perf_counter() - t0
    for prec in ('fp64', 'split-bf16'):
        call = lambda: lg.propagate_fft(lg.Wavefront(650e-9) * pl, wl.det_pixelscale,
                                        shape=wl.det_shape, oversample=wl.oversample,
                                        precision=prec).intensity_tensor()
        m_, p50_, p99_ = _timed(call, args.steps, args.warmup)
        fft_legs[prec] = {'value': 1e3 / m_, 'unit': 'PSFs/s', 'p50_ms': p50_, 'p99_ms': p99_,
                          'err_vs_oracle': lo.peak_normalised_error(call().cpu().numpy(), ref_fft)}
    fft_legs['cpu_baseline'] = {'value': 1.0 / cpu_fft_s, 'unit': 'PSFs/s', 'cores': os.cpu_count(),
                                'kind': kind, 'sample': f'one PSF through propagate_fft ({label})'}
    line = {'metric': 'monochromatic 256^2 PSFs/s', 'value': 1e3 / f_mean, 'unit': 'PSFs/s',
            'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': f_mean,
            'p50_ms': f_p50, 'p99_ms': f_p99, 'higher_is_better': True,
            'dtype': args.precision, 'data': 'synthetic (seeded)',
            'config': {'workload': 'monochromatic 256^2 circular pupil, Noll 2-11 N(0,20nm), '
                                   '650 nm, 128^2 detector x oversample 2',
                       'mft_tile': fused_tile},
            'path': 'PSFPlan.capture(...).replay() (the fused plan execute as a CUDA graph)',
            'fused_eager': {'value': 1e3 / e_mean, 'p50_ms': e_p50, 'p99_ms': e_p99,
                            'path': 'PSFPlan.execute'},
            'api_fp64': {'value': 1e3 / api_mean, 'p50_ms': api_p50, 'p99_ms': api_p99,
                         'err_vs_oracle': e_api},
            'err_vs_oracle': e_fused,
            'propagate_fft': fft_legs,
            'cpu_baseline': {'value': 1.0 / cpu_s, 'unit': 'PSFs/s', 'cores': os.cpu_count(),
                             'kind': kind, 'sample': f'5 PSFs through propagate_dft ({label})'}}
    print(json.dumps(line), flush=True)


def run_phase_retrieval(args):
    """512^2 circular pupil, OPD = Noll 2-37 N(0,30nm) + 18-segment PTT
    N(0,40nm), three images at defocus -1/0/+1 wave P-V (633 nm), 256^2
    detector x2: one loss + gradient evaluation per step."""
    import torch
    import lentil_gb300 as lg
    from lentil_gb300 import autodiff
    npix = 512
    amp = lg.normalize_power(lg.circle((npix, npix), npix // 2))
    support = amp > 0
    segs = lg.hex_segments(rings=2, seg_radius=116.8 * npix / 1024 * 1.0, seg_gap=2)
    segs = np.asarray([lg.pad(x, (npix, npix)) for x in segs]) * support
    basis, sigma = [], []
    rho, th = lg.zernike_coordinates(support)
    for j in range(2, 38):
        basis.append(lg.zernike(support, j, rho=rho, theta=th)); sigma.append(30e-9)
    for sg in segs:
        if sg.sum() == 0:
            continue
        r2, t2 = lg.zernike_coordinates(sg)
        for j in (1, 2, 3):
            basis.append(lg.zernike(sg, j, rho=r2, theta=t2)); sigma.append(40e-9)
    basis, sigma = np.asarray(basis), np.asarray(sigma)
    g = autodiff.geometry(amp, 633e-9, 1.0 / npix, 10.0, 5e-6, shape=256, oversample=2,
                          precision=args.precision)
    z4 = lg.zernike(support, 4)
    div = [k * 633e-9 / (z4.max() - z4.min()) * z4 for k in (-1, 0, 1)]
    rng = np.random.default_rng(4)
    true_c = rng.normal(0, 1, len(sigma)) * sigma
    pr = autodiff.PhaseRetrieval(amp, basis, div, [np.zeros(g.shape)] * 3, g)
    with torch.no_grad():
        t = [autodiff.mft_intensity(pr.opd(torch.as_tensor(true_c, device='cuda')) + d, pr.amp, g)
             for d in pr.diversity]
    pr.targets = [x + 1e-4 * x.max() * torch.as_tensor(rng.normal(size=g.shape), device='cuda')
                  for x in t]
    c = torch.zeros(len(sigma), dtype=torch.float64, device='cuda', requires_grad=True)

    def eager():
        c.grad = None
        pr.loss(c).backward()

    def step():                                     # loss + gradient replayed from CUDA graphs
        c.grad = None
        pr.graphed_loss(c).backward()

    e_mean, e_p50, e_p99 = _timed(eager, args.steps, args.warmup)
    mean, p50, p99 = _timed(step, args.steps, args.warmup)
    c.grad = None
    pr.graphed_loss(c).backward()
    g_graph = c.grad.clone()
    c.grad = None
    pr.loss(c).backward()
    grad_rel = float((g_graph - c.grad).abs().max() / c.grad.abs().max())
    pr.check()
    m, n = g.slc[2], g.slc[3]
    M, N = g.shape
    flops = 3 * 8.0 * (M * m * n + M * n * N) * 3      # forward + recompute + adjoint, 3 images
    line = {'metric': 'focus-diverse phase-retrieval loss+gradient evaluations/s',
            'value': 1e3 / mean, 'unit': 'evals/s', 'n_gpus': 1, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': mean, 'p50_ms': p50, 'p99_ms': p99,
            'higher_is_better': True, 'dtype': args.precision, 'data': 'synthetic (seeded)',
            'config': {'workload': '512^2 circular pupil, Noll 2-37 + 18-segment PTT, 3 diversity '
                                   'images at -1/0/+1 wave defocus, 633 nm, 256^2 detector x2',
                       'parameters': int(len(sigma)), 'mft_tile': tuner_summary(args),
                       'path': 'PhaseRetrieval.graphed_loss (forward and backward CUDA graphs)'},
            'eager': {'value': 1e3 / e_mean, 'p50_ms': e_p50, 'p99_ms': e_p99,
                      'path': 'PhaseRetrieval.loss (eager autograd)'},
            'graph_vs_eager_grad_rel_diff': grad_rel,
            'mft_tflops_algorithmic': flops / (mean / 1e3) / 1e12}
    print(json.dumps(line), flush=True)


def serving_requests(rng, grid, off_grid_fraction=0.0, server=None):
    """Seeded request generator of the serving mix: pupil 256/512/1024/2048,
    detector 64..1024 at oversample 2, 1-128 wavelengths over 400-1000 nm
    (on the server's grid, or, for ``off_grid_fraction`` of the requests,
    drawn uniformly and not on it), circular or 18-hex amplitude, Noll 2-11
    N(0, 20 nm) OPD.  With ``server``, the pupils and the Zernike bases are
    made resident on it once and each request carries its 10 coefficients;
    without, requests carry the amplitude and OPD arrays.  Returns
    make_request()."""
    import lentil_gb300 as lg
    from lentil_gb300 import serving
    pupils = {}
    for npix in (256, 512, 1024, 2048):
        circ = lg.normalize_power(lg.circle((npix, npix), npix // 2))
        segs = lg.hex_segments(rings=2, seg_radius=116.8 * npix / 1024, seg_gap=2)
        hexa = lg.normalize_power(lg.pad(np.sum(segs, axis=0), (npix, npix)))
        rho, th = lg.zernike_coordinates(circ > 0)
        basis = np.asarray([lg.zernike(circ > 0, j, rho=rho, theta=th) for j in range(2, 12)])
        if server is not None:
            pupils[npix] = (server.resident_pupil(circ), server.resident_pupil(hexa),
                            server.resident_basis(basis))
        else:
            pupils[npix] = (circ, hexa, basis)

    def make_request():
        npix = int(rng.choice([256, 512, 1024, 2048]))
        det = int(rng.choice([64, 128, 256, 512, 1024]))
        L = int(rng.integers(1, 129))
        circ, hexa, basis = pupils[npix]
        amp = circ if rng.random() < 0.5 else hexa
        coeffs = rng.normal(0, 20e-9, 10)
        if rng.random() < off_grid_fraction:
            wl = np.sort(rng.uniform(400e-9, 1000e-9, L))
            tag = 'off-grid'
        else:
            # L wavelengths spread over the server's 128-point 400-1000 nm grid
            idx = np.unique(np.linspace(0, len(grid) - 1, L).round().astype(int))
            wl = grid[idx]
            tag = 'grid'
        w = np.full(len(wl), 1.0 / len(wl))
        if server is not None:
            r = serving.PSFRequest(amp, coeffs, wl, w, 1.0 / npix, 10.0, 5e-6 * 1024 / npix, det,
                                   oversample=2, opd_basis=basis)
        else:
            r = serving.PSFRequest(amp, np.tensordot(coeffs, basis, 1), wl, w, 1.0 / npix, 10.0,
                                   5e-6 * 1024 / npix, det, oversample=2)
        r.tag = (tag, npix, det, len(wl))
        return r
    return make_request


def run_serving_rates(srv, make_request, rng, rates, duration, max_requests):
    """Poisson arrivals at each rate for ``duration`` seconds (at most
    ``max_requests``); per rate the latency, its split into queue wait
    (submit -> launch) and service (launch -> result), and the plan builds
    the window saw."""
    results, done = [], []
    for rate in rates:
        reqs = []
        t0 = time.perf_counter()
        t_next = t0
        while t_next - t0 < duration and len(reqs) < max_requests:
            now = time.perf_counter()
            if now < t_next:
                time.sleep(min(t_next - now, 0.002))
                continue
            r = make_request()
            srv.submit(r)
            reqs.append(r)
            t_next += rng.exponential(1.0 / rate)
        for r in reqs:
            r.future.result()
        t_end = max(r.t_done for r in reqs)
        lat = np.array([1e3 * r.latency for r in reqs])
        wait = np.array([1e3 * r.queue_wait for r in reqs if r.t_launch is not None])
        svc = np.array([1e3 * (r.t_done - r.t_launch) for r in reqs if r.t_launch is not None])
        window = [e for e in list(srv.events) if e[0] >= t0]
        builds = [e for e in window if e[1] == 'build']
        worst = sorted(reqs, key=lambda r: -r.latency)[:3]
        results.append({
            'rate_per_s': rate, 'requests': len(reqs), 'window_s': t_next - t0,
            'throughput_psfs_per_s': len(reqs) / (t_end - t0),
            'p50_ms': float(np.percentile(lat, 50)), 'p99_ms': float(np.percentile(lat, 99)),
            'queue_wait_p50_ms': float(np.percentile(wait, 50)) if len(wait) else None,
            'queue_wait_p99_ms': float(np.percentile(wait, 99)) if len(wait) else None,
            'service_p50_ms': float(np.percentile(svc, 50)) if len(svc) else None,
            'service_p99_ms': float(np.percentile(svc, 99)) if len(svc) else None,
            'plan_builds': len(builds), 'plan_build_ms': 1e3 * sum(e[2] for e in builds),
            'evictions': sum(1 for e in window if e[1] == 'evict'),
            'slowest': [{'latency_ms': 1e3 * r.latency, 'queue_wait_ms': 1e3 * (r.queue_wait or 0),
                         'request': list(r.tag)} for r in worst]})
        done.extend(reqs)
    return results, done


def serving_errors(done, precision, count=12, seed=9):
    """Peak-normalised error vs the complex128 plan of a seeded sample of
    served results (requests small enough for the FP64 form to finish in
    well under a second each)."""
    import torch
    import lentil_gb300 as lg
    rng = np.random.default_rng(seed)
    small = [r for r in done if r.tag[1] <= 1024 and r.tag[2] <= 512]
    pick = [small[i] for i in rng.choice(len(small), min(count, len(small)), replace=False)]
    errs = []
    for r in pick:
        got = r.future.result()
        amp = r.amp.tensor if hasattr(r.amp, 'tensor') else r.amp
        opd = r.opd
        if r.opd_basis is not None:             # the modal OPD, expanded in FP64 here
            opd = torch.tensordot(torch.as_tensor(r.opd, device='cuda'),
                                  r.opd_basis.tensor.double(), 1)
        pup = lg.Pupil(amplitude=amp, opd=opd, pixelscale=r.pixelscale_in,
                       focal_length=r.focal_length)
        ref = lg.broadband_psf(pup, r.wavelengths, r.weights, r.det_pixelscale,
                               shape=r.det_shape, oversample=r.oversample, precision='fp64')
        ref = ref.cpu().numpy() if hasattr(ref, 'cpu') else ref
        errs.append({'request': list(r.tag),
                     'err_vs_fp64': float(np.abs(got - ref).max() / np.abs(ref).max())})
    return {'sampled': len(errs), 'max': max(e['err_vs_fp64'] for e in errs) if errs else None,
            'median': float(np.median([e['err_vs_fp64'] for e in errs])) if errs else None,
            'results': errs}


def run_serving_leg(args):
    """Short serving leg of the default run (the serving mix of
    ``--workload serving`` at two rates after a warm pass): p50/p99 latency,
    throughput and the sampled error vs the complex128 form."""
    from lentil_gb300 import serving
    rng = np.random.default_rng(3)
    grid = np.linspace(400e-9, 1000e-9, 128)
    rates = [float(r) for r in args.serving_leg_rates.split(',')]
    with serving.PSFServer(streams=args.serve_streams, max_batch=args.serve_batch,
                           precision=args.precision, grid=grid) as srv:
        make_request = serving_requests(rng, grid, server=srv)
        run_serving_rates(srv, make_request, rng, [100.0], 4.0, 400)
        res, done = run_serving_rates(srv, make_request, rng, rates, 3.0, 600)
    errors = serving_errors(done, args.precision, count=6)
    return {'rates': res, 'err_vs_fp64_sampled': {k: errors[k] for k in ('sampled', 'max', 'median')},
            'workload': 'the serving mix (pupil 256-2048, detector 64-1024 x2, 1-128 '
                        'wavelengths on a 128-point grid, circular or 18-hex, Noll 2-11 '
                        'coefficients on resident pupils and bases), 3 s per rate after a '
                        '4 s warm pass at 100/s; serving_p50_ms/p99_ms are the first rate\'s'}


def run_serving(args):
    """Poisson stream of PSF requests: pupil 256/512/1024/2048, detector
    64..1024 at oversample 2, 1-128 wavelengths over 400-1000 nm, circular or
    18-hex amplitude, Noll 2-11 N(0,20nm) OPD; continuous batching server."""
    from lentil_gb300 import serving
    rng = np.random.default_rng(3)
    grid = np.linspace(400e-9, 1000e-9, 128)
    rates = [float(r) for r in args.rates.split(',')]
    with serving.PSFServer(streams=args.serve_streams, max_batch=args.serve_batch,
                           precision=args.precision, grid=grid) as srv:
        make_request = serving_requests(rng, grid, server=srv)
        # warm pass: every geometry's plan built and the tile widths tuned
        # before the measured rates (plan builds are reported per rate)
        warm, _ = run_serving_rates(srv, make_request, rng, [100.0], args.serve_warm, 400)
        results, done = run_serving_rates(srv, make_request, rng, rates, args.duration,
                                          args.max_requests)
        off = serving_requests(np.random.default_rng(4), grid, off_grid_fraction=0.1, server=srv)
        off_res, off_done = run_serving_rates(srv, off, rng, [200.0], args.duration,
                                              args.max_requests)
        raw = serving_requests(np.random.default_rng(5), grid)
        raw_res, _ = run_serving_rates(srv, raw, rng, [100.0], args.duration, args.max_requests)
        stats = dict(srv.stats)
    errors = serving_errors(done + off_done, args.precision)
    best = max(x['throughput_psfs_per_s'] for x in results)
    line = {'metric': 'serving mix PSFs/s with p50/p99 latency', 'value': best, 'unit': 'PSFs/s',
            'n_gpus': 1, 'higher_is_better': True, 'dtype': args.precision,
            'data': 'synthetic (seeded)', 'sweep': results, 'off_grid_10pct': off_res,
            'host_arrays_100_per_s': raw_res,
            'warm_pass': warm, 'err_vs_fp64_sampled': errors, 'server_stats': stats,
            'config': {'workload': 'Poisson PSF requests: pupil 256/512/1024/2048, detector '
                                   '64-1024 x oversample 2, 1-128 wavelengths on a 128-point '
                                   '400-1000 nm grid (off_grid_10pct: 10 % drawn off the grid), '
                                   'circular or 18-hex amplitude, Noll 2-11 N(0,20nm); pupils '
                                   'and Zernike bases resident on the server, requests carry '
                                   'coefficients (host_arrays_100_per_s: requests carrying '
                                   'amplitude and OPD arrays)',
                       'streams': args.serve_streams, 'max_batch': args.serve_batch,
                       'duration_s_per_rate': args.duration,
                       'max_requests_per_rate': args.max_requests,
                       'mft_tile': tuner_summary(args)}}
    print(json.dumps(line), flush=True)


def run_large(args):
    """4096^2 obscured 18-hex pupil with spiders, Noll 2-22 + 25 nm rms PSD,
    50 lambda/D tilt removed by fit_tilt (output shift), 32 wavelengths
    600-1000 nm, 1024^2 detector at oversample 4, then pixelate."""
    import torch
    import lentil_gb300 as lg
    from lentil_gb300 import broadband, workloads
    from oracle import lentil_oracle as lo
    npix = args.npix if args.npix != 1024 else 4096
    t0 = time.perf_counter()
    wl, mask, opd = workloads.large_segmented(npix=npix, n_wavelengths=32)
    pg = lg.Pupil(amplitude=wl.amp, opd=opd, pixelscale=wl.pixelscale_in, focal_length=10)
    pg.fit_tilt(inplace=True)
    prep_s = time.perf_counter() - t0
    s_, amp_eff, opd_fit = broadband.dense_field(pg)
    geo = broadband.plan_geometry(wl.plane_shape, s_, list(pg.tilt), pg.pixelscale, 10.0, lg.pupil,
                                  wl.wavelengths, wl.det_pixelscale, shape=wl.det_shape,
                                  oversample=wl.oversample)
    dev = torch.device('cuda', 0)
    A = torch.as_tensor(amp_eff[None], device=dev)
    O = torch.as_tensor(opd_fit[None], device=dev)
    W = torch.as_tensor(wl.weights[geo.keep][None], device=dev)
    out = torch.zeros((1,) + geo.shape_out, dtype=torch.float64, device=dev)
    plan = broadband.make_plan(geo, batch=1, precision=args.precision)

    def step():
        plan.execute(A, O, W, out=out, check=False)
        return lg.detector.pixelate(out[0], wl.oversample)

    mean, p50, p99 = _timed(step, args.steps, args.warmup)
    img = step().cpu().numpy()
    res = {'split_ms': mean, 'p50_ms': p50, 'p99_ms': p99}
    # pixelate alone (pixel MTF by FFT, then resampling): algorithmic bytes
    # 2 x (8 B read + 8 B write) per input pixel plus the decimated write
    pix_ms, _, _ = _timed(lambda: lg.detector.pixelate(out[0], wl.oversample), args.steps,
                          args.warmup)
    npx = out[0].numel()
    pix_bytes = 32 * npx + 8 * npx // wl.oversample ** 2
    pk, pk_kind = peaks()
    pix_gbs = pix_bytes / (pix_ms / 1e3) / 1e9
    t1 = time.perf_counter()
    plan64 = broadband.make_plan(geo, batch=1, precision='fp64')
    ref = torch.zeros_like(out)
    torch.cuda.synchronize()
    f0 = time.perf_counter()
    plan64.execute(A, O, W, out=ref)
    ref_img = lg.detector.pixelate(ref[0], wl.oversample).cpu().numpy()
    torch.cuda.synchronize()
    fp64_s = time.perf_counter() - f0
    del plan64
    err = lo.peak_normalised_error(img, ref_img)
    # CPU: lentil's loop on one wavelength (lentil itself where installed,
    # else the oracle port) after its own fit_tilt, scaled to 32, plus one
    # pixelate
    mod, kind, label = reference_module()
    po = mod.Pupil(amplitude=wl.amp, opd=opd.copy(), pixelscale=wl.pixelscale_in, focal_length=10)
    po.fit_tilt(inplace=True)                      # input preparation, as on the GPU side
    c0 = time.perf_counter()
    wf = mod.propagate_dft(mod.Wavefront(wl.wavelengths[0]) * po, wl.det_pixelscale,
                           shape=wl.det_shape, oversample=wl.oversample)
    one = wf.insert(np.zeros(wf.shape), weight=wl.weights[0])
    c1 = time.perf_counter()
    if hasattr(mod, 'detector'):
        mod.detector.pixelate(one, wl.oversample)
    else:
        mod.pixelate(one, wl.oversample)
    c2 = time.perf_counter()
    cpu_s = (c1 - c0) * len(wl.wavelengths) + (c2 - c1)
    m, n = geo.fslice[2], geo.fslice[3]
    M, N = geo.window_shape
    flops = 8.0 * (M * m * n + M * n * N) * len(geo.wavelengths)
    line = {'metric': 'large oversampled broadband pixelated PSFs/s', 'value': 1e3 / mean,
            'unit': 'PSFs/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': mean, 'p50_ms': p50, 'p99_ms': p99, 'higher_is_better': True,
            'dtype': args.precision, 'data': 'synthetic (seeded)',
            'config': {'workload': f'{npix}^2 obscured 18-hex pupil, 3 spiders, Noll 2-22 + '
                                   '25 nm PSD, 50 lambda/D tilt -> shift, 32 wavelengths '
                                   '600-1000 nm, 1024^2 detector x oversample 4, pixelate',
                       'field': [m, n], 'window': [M, N], 'tilt_shift_px': list(geo.shifts[0])},
            'err_vs_fp64': err, 'fp64_plain': {'seconds_per_psf': fp64_s,
                                               'speedup_split_over_fp64': fp64_s * 1e3 / mean},
            'mft_tflops_algorithmic': flops / (mean / 1e3) / 1e12,
            'pixelate_roofline': {'ms': pix_ms, 'algorithmic_bytes': pix_bytes,
                                  'achieved_gbs': pix_gbs, 'peak_gbs': pk.get('hbm_gbs', 6800.0),
                                  'frac': pix_gbs / pk.get('hbm_gbs', 6800.0),
                                  'peak_kind': f'{pk_kind} HBM copy',
                                  'path': 'detector.pixelate on the device image'},
            'input_prep_s': prep_s,
            'cpu_baseline': {'value': 1.0 / cpu_s, 'unit': 'PSFs/s', 'cores': os.cpu_count(),
                             'kind': kind, 'sample': f'1 of 32 wavelengths of lentil\'s loop '
                                                     f'({label}, after its fit_tilt), scaled to '
                                                     '32, plus one pixelate'}}
    print(json.dumps(line), flush=True)


def stage1_live_fraction(field_nonzero, width):
    """Fraction of the tensor-core stage 1's K blocks that are issued for a
    field (m x n nonzero pattern) at pair-tile width ``width``: a 64-wide K
    block covers two 32-row units of the field (the real rows, then the
    imaginary rows) and is skipped when both are zero across the whole
    column tile.  1.0 where the kernel tracks no flags (more than 128 K
    blocks)."""
    f = np.asarray(field_nonzero, dtype=bool)
    m, n = f.shape
    kp1, kp2 = -(-m // 32) * 32, -(-n // 32) * 32
    units = kp1 // 32                          # == K blocks of stage 1
    if units > 128:
        return 1.0
    g = np.zeros((kp1, kp2), dtype=bool)
    g[:m, :n] = f
    k = np.arange(units)
    tiles = -(-kp2 // width)
    live = 0
    for t in range(tiles):
        u = g[:, t * width:(t + 1) * width].reshape(units, 32, -1).any(axis=(1, 2))
        live += int(np.count_nonzero(u[(2 * k) % units] | u[(2 * k + 1) % units]))
    return live / (tiles * units)


def tuner_summary(args):
    """Tile width of this thread's last tensor-core launch and how it was chosen."""
    from lentil_gb300 import tuner
    how = {'measure': 'autotuner (online measurement)', 'model': 'autotuner (occupancy model)'}
    return {'last_tile': tuner.last_tile(), 'classes_decided': tuner.entries(),
            'chosen_by': f'forced --tile {args.tile}' if args.tile else how[args.tune]}


def main():
    args = parse()
    if args.impl != 'reference':
        from lentil_gb300 import tuner
        tuner.set_mode(args.tune)
        if args.tile:
            tuner.force_tile(args.tile)
    if args.workload == 'large':
        return run_large(args)
    if args.workload == 'serving':
        return run_serving(args)
    if args.impl == 'reference':
        run_reference(args)
    elif args.workload == 'monochromatic':
        run_monochromatic(args)
    elif args.workload == 'phase_retrieval':
        run_phase_retrieval(args)
    else:
        run_gpu(args)


if __name__ == '__main__':
    main()
