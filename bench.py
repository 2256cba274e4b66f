#!/usr/bin/env python
"""Benchmark of the flare render path: frames/s (and rays/s) of one full FLARE_STARBURST
frame of the 24-surface production workload on one GB300.

One step = one frame, nothing cached between frames: ghost aperture -> ghost FRFT texture,
ray trace (276 ghosts x 16 wavelengths x 128^2 grid = 72.4 M rays), quad and vertex setup,
tile binning, rasterisation into 2048 x 2048 RGBA, starburst aperture (8 blades, blurred
dust) -> diffraction spectrum -> starburst image, and the reference's composite
2 * flare + starburst.

* ``value``: frames/s with the inputs resident on the device (CUDA events on the stream).
* ``e2e``: the same frames through the public Engine API from a host-side Project to the
  host image (host->device inputs and the device->host image inside the timed region).
* ``cpu_baseline``: the reference's own kernels compiled for the host (oracle/_ref) on a
  bounded sample of the same frame, extrapolated per stage to a whole frame.
* ``--impl reference``: the reference arm, which times that CPU path per step.

Multi-GPU: each rank renders its own frames (replicas; the frame does not shard across
GPUs without an image reduce); ``value`` is the sum over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = 'production-24'
METRIC = 'frames/s (FLARE_STARBURST, 2048x2048, 276 ghosts x 16 wavelengths x 128^2 rays)'


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--workload', default=WORKLOAD)
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--cpu-whole-frames', action='store_true',
                    help='also measure a whole 16-surface CPU frame (about a minute) beside its sampled estimate')
    ap.add_argument('--no-e2e', action='store_true')
    # reductions of the workload for profiler captures (recorded in the line's config)
    ap.add_argument('--image', type=int, default=0, help='square image size override')
    ap.add_argument('--ghosts', type=int, default=0, help='keep only the first N ghosts')
    ap.add_argument('--batched-frames', type=int, default=256,
                    help='frames of the batched form measured beside the plain path (0 = skip)')
    ap.add_argument('--no-differentiable', action='store_true',
                    help='skip the forward+adjoint measurement of the 16-surface lens')
    ap.add_argument('--no-diagram', action='store_true',
                    help='skip the DIAGRAM element measurement (trace with hits and drawing)')
    ap.add_argument('--no-configs', action='store_true',
                    help='skip the 8- and 16-surface FLARE frames measured beside the production frame')
    ap.add_argument('--raster-stats', action='store_true',
                    help='count k_raster work (statistics build of the library) instead of timing')
    ap.add_argument('--differentiable-only', action='store_true',
                    help='only the forward+adjoint measurement of the 16-surface lens (for profiler captures)')
    return ap.parse_args()


def make_workload(args):
    from realflare_gb300 import synthetic
    from realflare_gb300.data import QSize

    w = synthetic.workload(args.workload)
    lens = w.project.flare.lens
    if args.image > 0:
        w.project.render.resolution = QSize(args.image, args.image)
    if args.ghosts > 0:
        lens.ghost_paths = lens.ghost_paths[:args.ghosts]
    return w


def workload_config(w, world: int) -> dict:
    """The line's config: the workload and its sizes (both arms report the same)."""
    from realflare_gb300 import prepare

    p = w.project
    ti = prepare.trace_inputs(p)
    a = ti.args
    r, sr = p.render.resolution, p.render.starburst.resolution
    return {
        'workload': w.name, 'image': f'{r.width()}x{r.height()}', 'ghosts': a.path_count,
        'wavelengths': a.wavelength_count, 'grid': a.grid_count, 'rays_per_frame': ti.ray_count,
        'starburst_aperture': f'{sr.width()}x{sr.height()}', 'parallelism': f'replicas{world}',
    }


def dist_init():
    import torch

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault('MASTER_ADDR', '127.0.0.1')
        dist.init_process_group('nccl' if torch.cuda.is_available() else 'gloo')
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    device = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, device: int) -> None:
        self.device = device
        self.proc = None
        self.path = None

    def start(self) -> None:
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', f'--id={self.device}', f'--query-gpu={self.FIELDS}', '--format=csv,noheader,nounits',
                 '-lms', '200'], stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        self.proc.wait()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(',')]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['no samples']}
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == 'active'})
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(rows)}


# ---------------------------------------------------------------------- GPU frame
class GpuFrame:
    """One FLARE_STARBURST frame from device-resident inputs, stage by stage."""

    STAGES = ('ghost', 'trace', 'setup', 'bin', 'raster', 'starburst', 'compose')

    def __init__(self, workload, flare_only: bool = False) -> None:
        import numpy as np
        import torch

        from realflare_gb300 import prepare
        from realflare_gb300._abi import lib
        from realflare_gb300.device import empty, to_device
        from realflare_gb300.tasks import RasterizingTask

        self.torch = torch
        self.lib = lib()
        self.w = workload
        p = workload.project
        self.p = p
        self.stream = torch.cuda.Stream()
        self.sh = int(self.stream.cuda_stream)
        ti = prepare.trace_inputs(p)
        self.ti = ti
        a = ti.args
        self.P, self.W, self.G = a.path_count, a.wavelength_count, a.grid_count
        self.R = self.G * self.G
        self.n_rays = ti.ray_count
        # resident inputs
        self.elements = to_device(ti.elements.view(np.uint8))
        self.paths = to_device(ti.paths)
        self.wavelengths = to_device(ti.wavelengths)
        gr = p.render.ghost.resolution
        self.gw, self.gh = gr.width(), gr.height()
        sr = p.render.starburst.resolution
        self.sw, self.sh_ = sr.width(), sr.height()
        d = p.flare.starburst_aperture.dust
        rng = np.random.Generator(np.random.PCG64(d.seed))
        self.noise = to_device(rng.random((self.sh_, self.sw), dtype=np.float32))
        # buffers
        self.rays = empty((6, self.n_rays))
        self.ghost_ap = empty((self.gh, self.gw))
        self.ghost = empty((self.gh, self.gw))
        self.frft_scratch = empty((3, self.gh, self.gw, 2))
        self.star_ap = empty((self.sh_, self.sw))
        self.blur_scratch = empty((self.sh_, self.sw))
        self.spectrum = empty((1, self.sh_, self.sw))
        self.spec_scratch = empty((2, 1, self.sh_, self.sw, 2))
        h, wd = p.render.resolution.height(), p.render.resolution.width()
        self.flare = empty((h, wd, 4))
        self.star = empty((h, wd, 4))
        self.out = empty((h, wd, 4))
        self.raster = RasterizingTask(self.stream)
        self.ra = prepare.raster_args(p, self.P, self.W, (self.gh, self.gw))
        self.area, self.min_area = prepare.quad_constants(p)
        from realflare_gb300.tasks import StarburstTask

        self.star_task = StarburstTask(self.stream)
        self.light = self.star_task.light()
        self.spectrum_tex = self.raster.spectrum()
        self.entries = 0
        self.events = None
        self.flare_only = flare_only

    def _ev(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e

    def step(self) -> None:
        import math

        from realflare_gb300._abi import StarburstArgs, check

        L, s, p = self.lib, self.sh, self.p
        ev = [self._ev()]
        # ghost aperture + FRFT texture
        ga = p.flare.ghost_aperture.shape
        check(L.rf_aperture_shape(self.ghost_ap.data_ptr(), self.gw, self.gh, ga.size.width(), ga.size.height(),
                                  ga.blades, math.radians(ga.rotation), ga.roundness, ga.softness / 10, s), 'shape')
        alpha = 0.15 * (560.0 / 400) * (p.flare.ghost.fstop / 18)
        check(L.rf_ghost_frft(self.ghost_ap.data_ptr(), self.gw, self.gh, alpha, self.frft_scratch.data_ptr(),
                              self.ghost.data_ptr(), s), 'frft')
        ev.append(self._ev())
        check(L.rf_trace(self.elements.data_ptr(), self.paths.data_ptr(), self.wavelengths.data_ptr(),
                         ctypes.byref(self.ti.args), self.rays.data_ptr(), s), 'trace')
        ev.append(self._ev())
        raster = self.raster
        Q = (self.G - 1) ** 2
        bounds = raster._buffer('bounds', self.P * Q * 4)
        inten = raster._buffer('intensities', self.P * Q * self.W)
        vtx = raster._buffer('vertexes', (self.n_rays + 1) * 8)
        check(L.rf_quad_setup(self.rays.data_ptr(), self.P, self.W, self.G, self.area, self.min_area,
                              bounds.data_ptr(), inten.data_ptr(), s), 'quad')
        check(L.rf_vertex(self.rays.data_ptr(), inten.data_ptr(), self.P, self.W, self.G, self.ra.screen_transform,
                          self.ra.width, self.ra.height, vtx.data_ptr(), s), 'vertex')
        ev.append(self._ev())
        with self.torch.cuda.stream(self.stream):
            offsets, entries = raster.bin(self.ra, bounds, vtx)
            order = raster.order(offsets)
        self.entries = raster.last_entry_count
        ev.append(self._ev())
        check(L.rf_raster_ordered(vtx.data_ptr(), offsets.data_ptr(), entries.data_ptr(), order.data_ptr(),
                                  self.ghost.data_ptr(), self.spectrum_tex.data_ptr(), ctypes.byref(self.ra),
                                  self.flare.data_ptr(), s), 'raster')
        ev.append(self._ev())
        if self.flare_only:  # a FLARE frame: no starburst, no composite
            ev += [self._ev(), self._ev()]
            self.events = ev
            return
        # starburst: aperture (shape x blurred dust), spectrum, compositor
        sa = p.flare.starburst_aperture
        check(L.rf_aperture_shape(self.star_ap.data_ptr(), self.sw, self.sh_, sa.shape.size.width(),
                                  sa.shape.size.height(), sa.shape.blades, math.radians(sa.shape.rotation),
                                  sa.shape.roundness, sa.shape.softness / 10, s), 'shape')
        check(L.rf_aperture_noise_dust(self.star_ap.data_ptr(), self.noise.data_ptr(), self.blur_scratch.data_ptr(),
                                       self.sw, self.sh_, sa.dust.strength, sa.dust.blur_sigma, s), 'dust')
        cfg = p.flare.starburst
        lam = (ctypes.c_float * 1)(560.0 * 1e-6)
        check(L.rf_starburst_spectrum(self.star_ap.data_ptr(), self.sw, self.sh_, lam, 1, max(1e-9, cfg.distance * 1e3),
                                      self.spec_scratch.data_ptr(), self.spectrum.data_ptr(), s), 'spectrum')
        a = StarburstArgs()
        h, wd = self.flare.shape[:2]
        a.width, a.height = wd, h
        a.spectrum_count, a.spectrum_height, a.spectrum_width = 1, self.sh_, self.sw
        a.samples = p.render.starburst.samples
        a.blur = cfg.blur / 100
        a.rotation = math.radians(cfg.rotation)
        a.rotation_weight = cfg.rotation_weight
        a.vignetting[0] = a.vignetting[1] = float('nan')
        a.intensity = cfg.intensity * 1e-6
        pos = p.flare.light.position
        a.offset[0], a.offset[1] = pos.x(), -pos.y()
        a.scale[0], a.scale[1] = cfg.scale.width(), cfg.scale.height() * wd / h
        a.lambda_first, a.lambda_step = 560.0, 1.0
        check(L.rf_starburst(self.spectrum.data_ptr(), self.light.data_ptr(), ctypes.byref(a), self.star.data_ptr(), s),
              'starburst')
        ev.append(self._ev())
        check(L.rf_axpby(self.flare.data_ptr(), 2.0, self.star.data_ptr(), 1.0, self.out.data_ptr(),
                         self.out.numel(), s), 'compose')
        ev.append(self._ev())
        self.events = ev

    def starburst_per_wavelength_ms(self, reps: int = 3) -> float:
        """Milliseconds of the starburst stage with one diffraction spectrum per rendered
        wavelength (16 FFTs over 390-700 nm, each sample reading the nearest wavelength's
        spectrum) instead of the reference's one spectrum at 560 nm: aperture, 16 spectra,
        compositor (CUDA events on the frame's stream, after one untimed run)."""
        import math

        from realflare_gb300._abi import StarburstArgs, check

        L, s, p = self.lib, self.sh, self.p
        wl = [float(x) for x in self.ti.wavelengths]
        n = len(wl)
        if not hasattr(self, '_spec_w'):
            self._spec_w = self.torch.empty((n, self.sh_, self.sw), device='cuda')
            self._spec_w_scratch = self.torch.empty((2, n, self.sh_, self.sw, 2), device='cuda')
        sa, cfg = p.flare.starburst_aperture, p.flare.starburst
        h, wd = self.flare.shape[:2]
        a = StarburstArgs()
        a.width, a.height = wd, h
        a.spectrum_count, a.spectrum_height, a.spectrum_width = n, self.sh_, self.sw
        a.samples = p.render.starburst.samples
        a.blur, a.rotation, a.rotation_weight = cfg.blur / 100, math.radians(cfg.rotation), cfg.rotation_weight
        a.vignetting[0] = a.vignetting[1] = float('nan')
        a.intensity = cfg.intensity * 1e-6
        pos = p.flare.light.position
        a.offset[0], a.offset[1] = pos.x(), -pos.y()
        a.scale[0], a.scale[1] = cfg.scale.width(), cfg.scale.height() * wd / h
        a.lambda_first, a.lambda_step = wl[0], (wl[-1] - wl[0]) / (n - 1) if n > 1 else 1.0
        lam = (ctypes.c_float * n)(*[x * 1e-6 for x in wl])

        def run():
            check(L.rf_aperture_shape(self.star_ap.data_ptr(), self.sw, self.sh_, sa.shape.size.width(),
                                      sa.shape.size.height(), sa.shape.blades, math.radians(sa.shape.rotation),
                                      sa.shape.roundness, sa.shape.softness / 10, s), 'shape')
            check(L.rf_aperture_noise_dust(self.star_ap.data_ptr(), self.noise.data_ptr(), self.blur_scratch.data_ptr(),
                                           self.sw, self.sh_, sa.dust.strength, sa.dust.blur_sigma, s), 'dust')
            check(L.rf_starburst_spectrum(self.star_ap.data_ptr(), self.sw, self.sh_, lam, n,
                                          max(1e-9, cfg.distance * 1e3), self._spec_w_scratch.data_ptr(),
                                          self._spec_w.data_ptr(), s), 'spectrum')
            check(L.rf_starburst(self._spec_w.data_ptr(), self.light.data_ptr(), ctypes.byref(a), self.star.data_ptr(),
                                 s), 'starburst')

        run()
        start = self._ev()
        for _ in range(reps):
            run()
        stop = self._ev()
        stop.synchronize()
        return start.elapsed_time(stop) / reps

    def accurate_trace_ms(self, reps: int = 3) -> float:
        """Milliseconds of rf_trace_accurate (double-precision ray geometry) on this frame's
        inputs, into the same ray buffer (CUDA events on the frame's stream, after one
        untimed run)."""
        from realflare_gb300._abi import check

        def run():
            check(self.lib.rf_trace_accurate(self.elements.data_ptr(), self.paths.data_ptr(),
                                             self.wavelengths.data_ptr(), ctypes.byref(self.ti.args),
                                             self.rays.data_ptr(), self.sh), 'rf_trace_accurate')

        run()
        start, stop = self._ev(), None
        for _ in range(reps):
            run()
        stop = self._ev()
        stop.synchronize()
        return start.elapsed_time(stop) / reps

    def stage_ms(self) -> dict:
        ev = self.events
        return {name: ev[i].elapsed_time(ev[i + 1]) for i, name in enumerate(self.STAGES)}


# ---------------------------------------------------------------------- CPU baseline
def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith('model name'):
                return line.split(':', 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open('/proc/cpuinfo') as f:
            for line in f:
                if line.lower().startswith('model name'):
                    return line.split(':', 1)[1].strip()
    except OSError:
        pass
    return 'unknown'


class CpuBaseline:
    """The reference's own kernels on the host cores (oracle/_ref, OpenMP over all cores;
    the C oracle when they are not built), timed on bounded samples of one frame.

    The whole frame's inputs (rays, primitives, vertices, bin masks, ghost texture,
    starburst spectrum) are computed once on the host, untimed. ``measure(seed)`` then
    times each stage on a sample and scales it to the whole frame:

    * trace: every k-th ghost (about 12), scaled by surface interactions (loop steps
      1 + elements + 2 (b1 - b2) per ray), since ghosts differ in length;
    * prim and vertex shaders on those ghosts' rays and the binner on their primitives,
      scaled by ghosts;
    * rasteriser: 64 stratified spans of 16 pixels (one at a seeded place in each cell of
      an 8 x 8 grid over the image), all in one parallel region, scaled by pixels;
    * starburst: a band of 32 rows at a seeded height, one parallel region, scaled by rows;
    * numpy FFT stages (starburst spectrum and ghost FRFT) whole.

    Different seeds draw different samples; their spread bounds the extrapolation error.
    """

    SPAN = 16
    CELLS = 8
    TRACE_GHOSTS = 12
    STAR_ROWS = 32

    def __init__(self, workload) -> None:
        import numpy as np

        from oracle import oracle as orc
        from realflare_gb300 import prepare
        from realflare_gb300.constants import light_spectrum

        self.np = np
        self.orc = orc
        self.prepare = prepare
        try:
            self.ref = orc.Reference()
            self.kind = 'reference'
        except (OSError, RuntimeError):
            self.ref, self.kind = None, 'port'
        self.o = orc.Oracle('f32')
        self.cpu = self.ref if self.ref is not None else self.o
        p = workload.project
        self.p = p
        ti = prepare.trace_inputs(p)
        self.ti = ti
        a = ti.args
        self.P, self.W, self.G = a.path_count, a.wavelength_count, a.grid_count
        self.R, self.Q = self.G ** 2, (self.G - 1) ** 2
        self.n_rays = self.P * self.W * self.R
        self.area, self.min_area = prepare.quad_constants(p)
        gr = p.render.ghost.resolution
        self.ra = prepare.raster_args(p, self.P, self.W, (gr.height(), gr.width()))
        self.spec = light_spectrum()
        self.threads = self.ref.set_threads(0) if self.ref is not None else os.cpu_count()
        # whole-frame inputs, untimed
        rays = self.trace_rays(ti)
        bounds, inten = self.o.quad_setup(rays, self.P, self.W, self.G, self.area, self.min_area)
        ra = self.ra
        self.vtx = self.o.vertex(rays, inten, self.P, self.W, self.G, ra.screen_transform, ra.width, ra.height)
        self.bounds = bounds
        self.masks = self.o.bin_masks(bounds, ra.screen_transform, ra.width, ra.height, ra.bin_size)
        del rays, inten
        ga = p.flare.ghost_aperture.shape
        self.ghost_ap = self.o.aperture_shape(gr.width(), gr.height(), (ga.size.width(), ga.size.height()),
                                              ga.blades, 0.0, ga.roundness, ga.softness / 10)
        self.ghost = orc.ghost_texture(self.ghost_ap, p.flare.ghost.fstop, self.ghost_ap.shape).astype(np.float32)
        sr = p.render.starburst.resolution
        sa = p.flare.starburst_aperture
        ap = self.o.aperture_shape(sr.width(), sr.height(), (sa.shape.size.width(), sa.shape.size.height()),
                                   sa.shape.blades, 0.0, sa.shape.roundness, sa.shape.softness / 10)
        if sa.dust.strength > 0 and sa.dust.blur_sigma > 0:
            rng = np.random.Generator(np.random.PCG64(sa.dust.seed))
            noise = rng.random((sr.height(), sr.width()), dtype=np.float32)
            ap = self.o.aperture_noise_dust(ap, noise, sa.dust.strength, sa.dust.blur_sigma)
        self.star_ap = ap
        self.fourier = orc.fft_power_spectrum(ap, 560e-6, max(1e-9, p.flare.starburst.distance * 1e3)).astype(
            np.float32)

    def trace_rays(self, ti):
        if self.ref is not None:
            return self.ref.trace(ti.elements, ti.paths, ti.wavelengths.astype(self.np.int32), ti.args)
        return self.o.trace(ti.elements, ti.paths, ti.wavelengths, ti.args)

    def starburst_args(self, h, w):
        from realflare_gb300._abi import StarburstArgs

        f = self.fourier
        sa = StarburstArgs()
        sa.width, sa.height = w, h
        sa.spectrum_width, sa.spectrum_height, sa.spectrum_count = f.shape[1], f.shape[0], 1
        sa.samples = self.p.render.starburst.samples
        sa.blur, sa.rotation, sa.rotation_weight = self.p.flare.starburst.blur / 100, 0.0, 1.0
        sa.vignetting[0] = sa.vignetting[1] = float('nan')
        sa.intensity = 1e-6
        sa.scale[0], sa.scale[1] = 1.0, 1.0
        sa.lambda_first, sa.lambda_step = 560.0, 1.0
        return sa

    def measure(self, seed: int = 0, small: bool = False) -> dict:
        """Per-stage seconds of one whole frame, extrapolated from this seed's samples.
        ``small`` shrinks every sample (for the one-thread figure)."""
        np, cpu, ti, prepare = self.np, self.cpu, self.ti, self.prepare
        ra = self.ra
        P, W, G = self.P, self.W, self.G
        out = {}
        # trace and setup: every k-th ghost, starting at a seeded offset
        n_ghosts = 2 if small else min(self.TRACE_GHOSTS, P)
        step = max(1, P // n_ghosts)
        sel = np.arange(seed % step, P, step)[:n_ghosts]
        sub = prepare.trace_inputs(self.p, paths=ti.paths[sel])
        t0 = time.perf_counter()
        rays = self.trace_rays(sub)
        t_trace = time.perf_counter() - t0
        out['trace'] = t_trace * trace_interactions(ti) / trace_interactions(sub)
        k = len(sel)
        t0 = time.perf_counter()
        if self.ref is not None:
            b, i = self.ref.prim_shader(rays, k, W, G, self.area, self.min_area)
            self.ref.vertex_shader(rays, i, k, W, G, ra.screen_transform, ra.width, ra.height)
            self.ref.binner(b, ra.screen_transform, ra.width, ra.height, ra.bin_size)
        else:
            b, i = self.o.quad_setup(rays, k, W, G, self.area, self.min_area)
            self.o.vertex(rays, i, k, W, G, ra.screen_transform, ra.width, ra.height)
            self.o.bin_masks(b, ra.screen_transform, ra.width, ra.height, ra.bin_size)
        out['setup_bin'] = (time.perf_counter() - t0) * P / k
        # raster: stratified spans in one parallel region
        h, w = ra.height, ra.width
        xy = self.orc.stratified_pixels(w, h, cells=self.CELLS, span=4 if small else self.SPAN, seed=seed)
        image = np.zeros((h, w, 4), np.float32)
        t0 = time.perf_counter()
        if self.ref is not None:
            self.ref.rasterizer_pixels(self.vtx, self.masks, self.ghost, self.spec, ra, xy, image)
        else:
            self.o.raster_pixels(self.vtx, self.masks, self.ghost, self.spec, ra, xy, image)
        out['raster'] = (time.perf_counter() - t0) * (h * w) / len(xy)
        # numpy FFT stages, whole
        t0 = time.perf_counter()
        self.orc.fft_power_spectrum(self.star_ap, 560e-6, max(1e-9, self.p.flare.starburst.distance * 1e3))
        self.orc.ghost_texture(self.ghost_ap, self.p.flare.ghost.fstop, self.ghost_ap.shape)
        out['fft'] = time.perf_counter() - t0
        # starburst: a band of rows
        rows = 1 if small else min(self.STAR_ROWS, h)
        y0 = int(np.random.default_rng(seed).integers(0, h - rows + 1))
        sa = self.starburst_args(h, w)
        t0 = time.perf_counter()
        cpu.starburst(self.fourier, self.spec, sa, rows=(y0, y0 + rows))
        out['starburst'] = (time.perf_counter() - t0) * h / rows
        return out

    def measure_one_thread(self) -> dict:
        """measure(small=True) with one OpenMP thread (the reference kernels only)."""
        if self.ref is None:
            return None
        previous = self.ref.set_threads(1)
        try:
            return self.measure(seed=0, small=True)
        finally:
            self.ref.set_threads(previous)

    def summary(self, samples: list, one_thread: dict | None = None) -> dict:
        """samples: per-seed stage seconds. value: frames/s of the median frame estimate."""
        totals = sorted(sum(st.values()) for st in samples)
        median = statistics.median(totals)
        stages = {k: statistics.median(st[k] for st in samples) for k in samples[0]}
        out = {
            'value': 1.0 / median,
            'unit': 'frames/s',
            'cores': self.threads,
            'cpu_model': cpu_model(),
            'kind': self.kind,
            'build': 'g++/gcc -O3 -fopenmp -ffp-contract=off (no -march=native: one source for x86 and Arm)',
            'sample': (f'one frame of this workload per seed ({len(samples)} seeds): trace of every k-th ghost '
                       f'({min(self.TRACE_GHOSTS, self.P)} of {self.P}) scaled by surface interactions, prim/vertex '
                       f'shaders and binner on their primitives scaled by ghosts, rasteriser on '
                       f'{self.CELLS * self.CELLS} stratified spans of {self.SPAN} pixels in one parallel region '
                       f'scaled by pixels, starburst on {self.STAR_ROWS} rows, numpy FFT stages whole'),
            'stage_seconds': {k: round(v, 3) for k, v in stages.items()},
            'frame_seconds_per_seed': [round(t, 2) for t in totals],
            'spread': round((totals[-1] - totals[0]) / median, 4),
            'rays_per_s': self.n_rays / stages['trace'],
        }
        if one_thread is not None:
            t1 = sum(one_thread.values())
            out['one_thread'] = {'value': 1.0 / t1, 'unit': 'frames/s', 'cores': 1,
                                 'stage_seconds': {k: round(v, 2) for k, v in one_thread.items()},
                                 'sample': '2 ghosts traced, 64 spans of 4 pixels, 1 starburst row'}
        return out


def whole_frame_check(name: str) -> dict:
    """One whole frame of a flare-only workload (8-surface, or 16-surface) with the
    reference's kernels on all host cores, stage by stage, beside the sampled estimate of
    the same frame: the measured extrapolation error."""
    import numpy as np

    from oracle import oracle as orc
    from realflare_gb300 import synthetic

    w = synthetic.workload(name, integer_wavelengths=True)
    base = CpuBaseline(w)
    cpu, ra = base.cpu, base.ra
    t0 = time.perf_counter()
    rays = base.trace_rays(base.ti)
    t_trace = time.perf_counter() - t0
    t0 = time.perf_counter()
    if base.ref is not None:
        b, i = base.ref.prim_shader(rays, base.P, base.W, base.G, base.area, base.min_area)
        v = base.ref.vertex_shader(rays, i, base.P, base.W, base.G, ra.screen_transform, ra.width, ra.height)
        m = base.ref.binner(b, ra.screen_transform, ra.width, ra.height, ra.bin_size)
    else:
        b, i = base.o.quad_setup(rays, base.P, base.W, base.G, base.area, base.min_area)
        v = base.o.vertex(rays, i, base.P, base.W, base.G, ra.screen_transform, ra.width, ra.height)
        m = base.o.bin_masks(b, ra.screen_transform, ra.width, ra.height, ra.bin_size)
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    if base.ref is not None:
        base.ref.rasterizer(v, m, base.ghost, base.spec, ra)
    else:
        base.o.raster(v, m, base.ghost, base.spec, ra)
    t_raster = time.perf_counter() - t0
    whole = t_trace + t_setup + t_raster
    est = [base.measure(seed) for seed in range(4)]
    est_flare = [e['trace'] + e['setup_bin'] + e['raster'] for e in est]
    return {
        'workload': name, 'kind': base.kind, 'cores': base.threads,
        'rays': base.n_rays, 'image': f'{ra.width}x{ra.height}',
        'measured_seconds': {'trace': round(t_trace, 3), 'setup_bin': round(t_setup, 3),
                             'raster': round(t_raster, 3), 'flare': round(whole, 3)},
        'measured_frames_per_s': 1.0 / whole, 'measured_rays_per_s': base.n_rays / t_trace,
        'sampled_flare_seconds': [round(x, 3) for x in est_flare],
        'sampled_over_measured': round(statistics.median(est_flare) / whole, 4),
    }


# ---------------------------------------------------------------------- main
def load_peaks() -> tuple:
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


def raster_profile(kernel: str = 'k_raster') -> dict:
    """Figures of a kernel on the production frame from its committed ncu summary
    (k_raster: DRAM bytes of one launch, tile entries and fragments of that launch;
    k_trace: issue-slot use on the reduced case)."""
    path = os.path.join(ROOT, 'profiles', f'{kernel}_production-24.json')
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def trace_interactions(ti) -> int:
    """Surface interactions of a trace: per ray that reaches the sensor, the reference's
    loop steps 1 + elements + 2 (b1 - b2) (raytracing.cl:258-352), summed over every ray."""
    paths = ti.paths.astype('int64')
    per_ray = 1 + ti.args.element_count + 2 * (paths[:, 0] - paths[:, 1])
    return int(per_ray.sum()) * ti.args.wavelength_count * ti.args.grid_count ** 2


# FP32 operations of the reference's trace arithmetic (realflare/api/tasks/cl/raytracing.cl,
# as written: no fused multiply-adds; add, subtract, multiply, divide, square root and each
# sin/cos/tan/asin/acos call count 1; comparisons, min/max, abs and negation 0). The
# refractive index of a (wavelength, element) is one value per frame, so dispersion is not
# counted per interaction.
TRACE_FLOPS = {
    'intersect_sphere': 59,   # intersect 123-175 with the incidence acos (sphere)
    'intersect_flat': 8,      # intersect, flat element
    'aperture': 2,            # pos_apt = pos.xy / height
    'rrel': 5,                # max(rrel, length(pos.xy) / height)
    'refract': 26,            # n1 / n2 and refract 70-86
    'reflect': 14,            # reflect 96-102, theta = incident + 1e-9, reflectance *= R
    'fresnel': 24,            # fresnel 1-16 (uncoated)
    'fresnel_ar': 77,         # nc, d1 and fresnel_ar 18-59 (single layer)
    'two_layer': 149,         # the exact two-layer stack (no reference counterpart)
    'init': 20,               # grid point, normalize(-direction), back-off (plus the intersect)
}
# One fragment of the rasteriser (covered pixel x record): compute_barycentric_quad
# (rasterizing.cl:95-148) 67, fragment_shader (471-506) times the hits 71, the colour lookup
# and accumulation (640-650) 12, counted the same way.
RASTER_FRAGMENT_FLOPS = 150
# The same fragment as the fewest instructions (multiply-adds fused, reciprocal, rsqrt and
# floor one each, the record's per-corner terms set up once per record): mean-value weights
# 68, fragment 49 (four of them the texel loads).
RASTER_FRAGMENT_MIN_INSTRUCTIONS = 117


def trace_flops(ti) -> int:
    """FP32 operations of a whole trace, every ray completing its path (TRACE_FLOPS per loop
    step, walking each ghost path's element sequence by the reference's loop rules,
    raytracing.cl:258-352)."""
    el = ti.elements
    E, apt = ti.args.element_count, ti.args.aperture_index
    R = ti.args.grid_count ** 2
    f = TRACE_FLOPS
    total = 0
    for b1, b2 in ti.paths.astype(int):
        ops = f['init'] + (f['intersect_sphere'] if el['radius'][0] != 0 else f['intersect_flat'])
        step, delta, i = 0, 1, 0
        while 0 <= i < E:
            ops += f['intersect_sphere'] if el['radius'][i] != 0 else f['intersect_flat']
            if i == apt:
                ops += f['aperture']
            else:
                ops += f['rrel']
                if i != E - 1:
                    if (step == 0 and i == b1) or (step == 1 and i == b2):
                        step += 1
                        delta = -delta
                        ops += f['reflect']
                        if el['coating_layers'][i] == 2:
                            ops += f['two_layer']
                        elif el['coating_layers'][i] == 1 or el['coating'][i] > 0:
                            ops += f['fresnel_ar']
                        else:
                            ops += f['fresnel']
                    else:
                        ops += f['refract']
            i += delta
        total += ops
    return total * ti.args.wavelength_count * R


def fp32_peak_tflops() -> float:
    """Derived FP32 peak: SMs x 128 FP32 lanes x 2 (multiply-add) x the measured maximum SM
    clock of this pool (MEASURED_PEAKS.json sm_max_mhz, else 2070 MHz)."""
    mhz = 2070.0
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as fh:
            mhz = float(json.load(fh).get('sm_max_mhz', mhz))
    except (OSError, ValueError):
        pass
    sms = 152
    try:
        import torch

        if torch.cuda.is_available():
            sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    return sms * 128 * 2 * mhz * 1e6 / 1e12


def issue_peak_ginstr() -> float:
    """Instruction issue peak in thread instructions per second (G): SMs x 4 schedulers x 32
    lanes x the maximum SM clock (one warp instruction per scheduler per cycle)."""
    return fp32_peak_tflops() * 1e3 / 2.0


def run_reference(args, rank, world) -> None:
    """The reference arm: each step is one frame estimate from a seeded sample (the seeds
    differ between steps) of the reference's kernels on all host cores."""
    if rank != 0:
        return
    w = make_workload(args)
    cpu = CpuBaseline(w)
    samples, times = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        st = cpu.measure(seed=i)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
            samples.append(st)
    s = cpu.summary(samples)
    line = {
        'impl': 'reference', 'metric': METRIC,
        'value': s['value'], 'unit': 'frames/s', 'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1e3 / s['value'], 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32', 'data': 'synthetic',
        'config': workload_config(w, args.gpus),
        'cpu_baseline': {k: s[k] for k in ('value', 'unit', 'cores', 'kind', 'sample', 'cpu_model', 'build',
                                           'spread', 'frame_seconds_per_seed')},
        'e2e': {'value': s['value'], 'unit': 'frames/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
        'stage_seconds': s['stage_seconds'], 'rays_per_s': s['rays_per_s'],
        'sample_wall_s': statistics.median(times) if times else None,
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    args = parse_args()
    rank, world = dist_init()
    if args.impl == 'reference':
        run_reference(args, rank, world)
        return
    if args.raster_stats:
        run_raster_stats(args)
        return
    if args.differentiable_only:
        print(json.dumps({'differentiable': run_differentiable(args)}), flush=True)
        return
    import torch

    from realflare_gb300._abi import lib

    w = make_workload(args)
    frame = GpuFrame(w)
    for _ in range(max(args.warmup, 3)):
        frame.step()
    torch.cuda.synchronize()
    L = lib()
    clocks = Clocks(torch.cuda.current_device())
    barrier(world)
    torch.cuda.synchronize()
    launches0 = L.rf_launch_count()
    clocks.start()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record(frame.stream)
    for _ in range(args.steps):
        frame.step()
    stop.record(frame.stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(world)
    launches = L.rf_launch_count() - launches0
    elapsed = start.elapsed_time(stop) / 1e3
    # per-stage times of the last timed step (events of every stage are recorded each step)
    last = frame.stage_ms()
    elapsed = max_over_ranks(elapsed, world)
    fps = args.steps / elapsed * world

    trace_accurate_ms = frame.accurate_trace_ms() if rank == 0 else None
    star_w_ms = frame.starburst_per_wavelength_ms() if rank == 0 else None
    # e2e through the Engine API: host Project in, host image out
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(w, args)
    batched = run_batched(args) if args.batched_frames > 0 and rank == 0 else None
    differentiable = run_differentiable(args) if not args.no_differentiable and rank == 0 else None
    diagram = run_diagram(args) if not args.no_diagram and rank == 0 else None
    configs = run_configs(args) if not args.no_configs and rank == 0 else None

    peak, peak_kind = load_peaks()
    raster_s = last['raster'] / 1e3
    entries = frame.entries
    h, wd = frame.flare.shape[:2]
    alg_bytes = entries * (4 + 4 * 64) + h * wd * 16
    achieved = alg_bytes / raster_s / 1e9
    prof = raster_profile()
    trace_prof = raster_profile('k_trace')
    interactions = trace_interactions(frame.ti)
    flops = trace_flops(frame.ti)
    traffic = fragments = None
    if prof.get('workload') == args.workload and prof.get('tile_entries') == entries:
        # the summary was taken on this very launch (same workload, same tile entries)
        traffic = prof['dram_bytes']
        fragments = prof['fragments']
    roofline = {
        'kernel': 'k_raster', 'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
        'frac': achieved / peak, 'peak_source': f'{peak_kind} hbm_gbs',
        'traffic': traffic,
        'algorithmic_bytes': alg_bytes,
        'fragments_per_s': fragments / raster_s if fragments else None,
        # the bound that limits this kernel: instruction issue (ncu on the reduced case)
        'issue_active': prof.get('issue_active_small'),
        'issue': {
            'bound': 'issue', 'unit': 'G thread-instructions/s',
            'achieved': fragments * RASTER_FRAGMENT_MIN_INSTRUCTIONS / raster_s / 1e9 if fragments else None,
            'peak': issue_peak_ginstr(),
            'frac': (fragments * RASTER_FRAGMENT_MIN_INSTRUCTIONS / raster_s / 1e9 / issue_peak_ginstr()
                     if fragments else None),
            'instructions_per_fragment': RASTER_FRAGMENT_MIN_INSTRUCTIONS,
            'note': ('the fewest instructions of one fragment of the reference arithmetic (multiply-adds fused) x '
                     'fragments / time, against one warp instruction per scheduler per cycle at the maximum '
                     'clock (derived)'),
        },
        'fp32': {
            'bound': 'fp32', 'unit': 'TFLOP/s',
            'achieved': fragments * RASTER_FRAGMENT_FLOPS / raster_s / 1e12 if fragments else None,
            'peak': fp32_peak_tflops(),
            'frac': fragments * RASTER_FRAGMENT_FLOPS / raster_s / 1e12 / fp32_peak_tflops() if fragments else None,
            'flops_per_fragment': RASTER_FRAGMENT_FLOPS,
            'note': 'FP32 peak derived: SMs x 128 lanes x 2 x maximum SM clock (none is measured in MEASURED_PEAKS.json)',
        },
        'note': ('issue-bound per-fragment shading (mean-value weights, bilinear ghost lookup per covered '
                 'pixel x record): issue_active is the fraction of cycles the warp schedulers issue an '
                 'instruction (ncu smsp__issue_active, 1024^2 / 48-ghost case of the same kernel); the vertex '
                 'reads hit L2, so DRAM traffic is far below the algorithmic bytes'),
    }
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        base = CpuBaseline(w)
        cpu = base.summary([base.measure(seed) for seed in range(4)], base.measure_one_thread())
        del base
        cpu['whole_frame_check'] = [whole_frame_check('plain-8')]
        if args.cpu_whole_frames:
            cpu['whole_frame_check'].append(whole_frame_check('spectral-16'))
    if rank == 0:
        line = {
            'metric': METRIC,
            'value': fps, 'unit': 'frames/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': elapsed / args.steps * 1e3, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': workload_config(w, world),
            'l2': (f'per-frame working set (rays {frame.rays.numel() * 4 / 1e9:.2f} GB, tile entries '
                   f'{entries * 4 / 1e9:.2f} GB) > L2 (129 MB): inputs larger than L2, no flush'),
            'rays_per_s': frame.n_rays / (last['trace'] / 1e3) * world,
            # k_trace: FP32 / issue-bound (no DRAM or tensor bound applies)
            'trace': {
                'rays_per_s': frame.n_rays / (last['trace'] / 1e3) * world,
                'surface_interactions': interactions,
                'surface_interactions_per_s': interactions / (last['trace'] / 1e3) * world,
                'issue_active': trace_prof.get('issue_active_small'),
                'flops': flops,
                'flops_per_interaction': flops / interactions,
                'fp32_tflops': flops / (last['trace'] / 1e3) / 1e12 * world,
                'fp32_peak_tflops': fp32_peak_tflops(),
                'fp32_frac': flops / (last['trace'] / 1e3) / 1e12 / fp32_peak_tflops(),
                'accurate_ms': trace_accurate_ms,
                'accurate_frame_ms': (elapsed / args.steps * 1e3 - last['trace'] + trace_accurate_ms
                                      if trace_accurate_ms else None),
                'note': ('interactions: 1 + elements + 2 (b1 - b2) loop steps per ray that reaches the sensor; '
                         'issue_active: ncu smsp__issue_active of k_trace, 1024^2 / 48-ghost case; accurate_ms: '
                         'rf_trace_accurate (double-precision ray geometry) on the same frame'),
            },
            'stage_ms': {k: round(v, 3) for k, v in last.items()},
            # the configuration's wording: the starburst "FFT-diffracted per wavelength and
            # composited" (16 spectra) instead of the reference's one spectrum at 560 nm
            'starburst_per_wavelength': {
                'wavelengths': len(frame.ti.wavelengths), 'stage_ms': star_w_ms,
                'frame_ms': elapsed / args.steps * 1e3 - last['starburst'] + star_w_ms if star_w_ms else None,
            },
            'tile_entries': entries,
            'e2e': e2e,
            'roofline': roofline,
            'cpu_baseline': cpu,
            'clocks': clk,
            'gpu_launches': launches,
            'batched': batched,
            'differentiable': differentiable,
            'diagram': diagram,
            'configs': configs,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_configs(args, steps: int = 20) -> dict:
    """FLARE frames (ghost texture, trace, setup, binning, raster; no starburst) of the
    8-surface workload (512^2, 28 ghosts, 32^2 grid, 1 wavelength) and the 16-surface
    workload (1024^2, 120 ghosts, 64^2 grid, 8 wavelengths) with device-resident inputs:
    frames/s and rays/s (CUDA events over ``steps`` frames after 3 warm-up frames)."""
    import torch

    from realflare_gb300 import synthetic

    out = {}
    for name in ('plain-8', 'spectral-16'):
        frame = GpuFrame(synthetic.workload(name), flare_only=True)
        for _ in range(3):
            frame.step()
        torch.cuda.synchronize()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(frame.stream)
        trace_ms = []
        for _ in range(steps):
            frame.step()
            trace_ms.append(frame.events)
        stop.record(frame.stream)
        torch.cuda.synchronize()
        seconds = start.elapsed_time(stop) / 1e3 / steps
        t_trace = statistics.median(ev[1].elapsed_time(ev[2]) for ev in trace_ms) / 1e3
        stage = frame.stage_ms()
        out[name] = {
            'image': f'{frame.ra.width}x{frame.ra.height}', 'ghosts': frame.P, 'wavelengths': frame.W,
            'grid': frame.G, 'rays': frame.n_rays, 'frames_per_s': 1.0 / seconds, 'ms_per_frame': seconds * 1e3,
            'rays_per_s': frame.n_rays / t_trace,
            'stage_ms': {k: round(v, 4) for k, v in stage.items() if k not in ('starburst', 'compose')},
        }
        del frame
    return out


def run_raster_stats(args) -> None:
    """One frame with the product library, then its raster pass again through the statistics
    build, which counts record iterations per 8 x 4 block and fragments (covered pixel x
    record pairs)."""
    import ctypes

    import torch

    from realflare_gb300 import build as rf_build
    from realflare_gb300._abi import SIGNATURES

    frame = GpuFrame(make_workload(args))
    frame.step()
    torch.cuda.synchronize()
    S = ctypes.CDLL(rf_build.build(stats=True))
    S.rf_raster.argtypes = SIGNATURES['rf_raster']
    S.rf_raster.restype = ctypes.c_int
    S.rf_raster_stats.argtypes = [ctypes.POINTER(ctypes.c_ulonglong)]
    S.rf_raster_stats.restype = ctypes.c_int
    out = (ctypes.c_ulonglong * 8)()
    assert S.rf_raster_stats(out) == 0
    r = frame.raster
    st = S.rf_raster(r._buffers['vertexes'].data_ptr(), r._buffers['tile_offsets'].data_ptr(),
                     r._buffers['tile_entries'].data_ptr(), frame.ghost.data_ptr(), frame.spectrum_tex.data_ptr(),
                     ctypes.byref(frame.ra), frame.flare.data_ptr(), frame.sh)
    torch.cuda.synchronize()
    assert st == 0, st
    assert S.rf_raster_stats(out) == 0
    it, whole, frag, frag_whole, blocks, frag_zero, iter_zero, steps = (int(v) for v in out)
    h, wd = frame.flare.shape[:2]
    print(json.dumps({
        'raster_stats': {
            'tile_entries': frame.entries, 'block_visits': blocks, 'record_iterations': it,
            'whole_block_record_iterations': whole, 'fragments': frag, 'fragments_in_whole_blocks': frag_whole,
            'fragments_per_pixel': frag / (h * wd), 'lane_efficiency': frag / max(1, 32 * it),
            'shading_steps': steps, 'step_lane_efficiency': frag / max(1, 32 * steps) if steps else None,
        },
        'config': {'workload': args.workload, 'image': f'{wd}x{h}', 'ghosts': frame.P},
    }), flush=True)


def run_batched(args) -> dict:
    """The batched form against per-frame plain launches on the same frames: 256 requests
    (lenses with 8/16/24 surfaces, 32^2/64^2/128^2 grids, 1-16 wavelengths, lights uniform
    over the field) at 1024^2. Frames are grouped under a device-memory budget; each group
    is one launch per stage, captured as one CUDA graph and replayed (timed). The plain
    path renders frame by frame through the task API (trace, setup, bin with its host
    synchronisation, raster). Both are timed from a synchronised start to a synchronised
    end; the images are compared bit for bit."""
    import numpy as np
    import torch

    from realflare_gb300 import synthetic
    from realflare_gb300.autotune import autotune
    from realflare_gb300.batch import BatchRenderer, ghost_textures, group_frames
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    n = args.batched_frames
    projects = synthetic.batched_projects(n, seed=0, resolution=1024)
    ghosts = ghost_textures(projects)
    tex, offsets, shapes = ghosts
    free, _ = torch.cuda.mem_get_info()
    budget = int(min(0.3 * free, 60e9))
    groups = group_frames(projects, budget)
    # autotune on a sample spread over the batch (the knobs do not change the images)
    sample = projects[:: max(1, n // 24)][:24]
    choice = autotune(sample)

    # batched: per group build, size and capture (untimed), then time the graph replays
    batched_s, sums_batched = 0.0, []
    for g in groups:
        r = BatchRenderer([projects[i] for i in g], tile_size=choice.tile_size,
                          rays_per_thread=choice.rays_per_thread, ghosts=(tex, [offsets[i] for i in g],
                                                                         [shapes[i] for i in g]))
        r.run()
        r.capture()
        r.replay()  # warm
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.replay()
        torch.cuda.synchronize()
        batched_s += time.perf_counter() - t0
        sums_batched += [float(im.double().sum()) for im in r.images]
        del r
    # plain: frame after frame through the task API
    trace, raster = RaytracingTask(cache=False), RasterizingTask()
    for p in projects[:2]:  # warm-up
        raster.run(p, trace.run(p), Image(tensor=tex[offsets[0]: offsets[0] + shapes[0][0] * shapes[0][1]]
                                          .view(*shapes[0])))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    images = []
    for i, p in enumerate(projects):
        h, w = shapes[i]
        img = raster.run(p, trace.run(p), Image(tensor=tex[offsets[i]: offsets[i] + h * w].view(h, w)))
        images.append(img.tensor.double().sum())
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    sums_plain = [float(x) for x in images]
    identical = bool(np.array_equal(np.array(sums_batched), np.array(sums_plain)))
    rays = sum(p.render.grid_count ** 2 * p.render.wavelength_count * len(p.flare.lens.ghost_paths)
               for p in projects)
    return {
        'frames': n, 'image': '1024x1024', 'rays': rays,
        'frames_per_s': n / batched_s, 'plain_frames_per_s': n / plain_s, 'speedup_vs_plain': plain_s / batched_s,
        'groups': len(groups), 'memory_budget_gb': round(budget / 1e9, 1),
        'tile_size': choice.tile_size, 'rays_per_thread': choice.rays_per_thread,
        'autotune_ms': {k: round(v, 3) for k, v in choice.timings_ms.items()},
        'identical_to_plain': identical,
        'timing': 'wall clock from a synchronised start to a synchronised end; batched = CUDA-graph replays',
    }


def run_differentiable(args) -> dict:
    """Forward+adjoint against the plain forward on the 16-surface lens at 512^2 (64^2 grid,
    8 wavelengths, 120 ghosts), gradients with respect to 16 radii, 15 gaps, 16 coating
    thicknesses and 2 light coordinates; then 200 Adam steps of parameter recovery."""
    import torch

    from realflare_gb300 import synthetic
    from realflare_gb300.diff import DifferentiableRenderer
    from realflare_gb300.recover import recover
    from realflare_gb300.tasks import GhostApertureTask, GhostTask

    w = synthetic.workload('differentiable-16')
    p = w.project
    ghost = GhostTask().run(p, GhostApertureTask().run(p)).tensor
    r = DifferentiableRenderer(p, ghost)
    params = [t.clone().requires_grad_(True) for t in r.params.tensors()]
    target = torch.zeros((p.render.resolution.height(), p.render.resolution.width(), 4), device='cuda')

    def forward():
        with torch.no_grad():
            radius, center, t, direction = r.params.elements(*params, r.E)
            return r.forward_kernels(radius, center, t, direction)

    def forward_adjoint():
        for q in params:
            q.grad = None
        image = r.render(*params)
        ((image - target)[..., :3] ** 2).sum().backward()

    def timed(fn, n=10):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / n * 1e3

    f_ms = timed(forward)
    fa_ms = timed(forward_adjoint)
    rec = recover(p, ghost, steps=200)
    return {
        'workload': 'differentiable-16', 'image': '512x512', 'rays': r.n_rays,
        'parameters': sum(q.numel() for q in params),
        'forward_ms': f_ms, 'forward_adjoint_ms': fa_ms, 'ratio': fa_ms / f_ms,
        'recovery': {'coarse_steps': rec.coarse_steps, 'image_steps': rec.steps,
                     'loss_initial': rec.loss_initial, 'loss_before_image_stage': rec.loss_start,
                     'loss_end': rec.loss_end, 'param_rms_error_start': rec.error_start,
                     'param_rms_error_after_coarse': rec.error_after_coarse, 'param_rms_error_end': rec.error_end,
                     'group_rms_error_start': rec.error_groups_start, 'group_rms_error_end': rec.error_groups_end,
                     'seconds': rec.seconds,
                     'stages': ('coarse: blurred ray splat against the blurred target (blur 8, 4, 2, 1 px); image: '
                                '200 Adam steps of the image loss over the coating thicknesses')},
        'timing': 'wall clock per iteration (each includes the binning host synchronisation)',
    }


def run_diagram(args) -> dict:
    """The DIAGRAM element at the reference's default diagram settings (2048 x 1024, 8 x 8
    grid, grid length 50, one ghost) on the workload's lens: GPU milliseconds per render (the
    trace with every hit stored, then the drawing; CUDA events on the tasks' stream, inputs
    uploaded each render), and the reference's own kernels (oracle/_ref, else the C
    oracle) on the same inputs on the host cores."""
    import numpy as np
    import torch

    from oracle import oracle as orc
    from realflare_gb300 import prepare, synthetic
    from realflare_gb300.tasks import DiagramTask, IntersectionsTask

    p = synthetic.workload(args.workload).project
    d = p.diagram
    stream = torch.cuda.Stream()
    inter_task, draw_task = IntersectionsTask(stream), DiagramTask(stream)

    def render():
        with torch.cuda.stream(stream):
            return draw_task.run(p, inter_task.run(p, (d.debug_ghost,)))

    for _ in range(3):
        image = render()
    n = 20
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream.synchronize()
    start.record(stream)
    for _ in range(n):
        render()
    end.record(stream)
    end.synchronize()
    gpu_ms = start.elapsed_time(end) / n
    got = image.tensor.cpu().numpy()

    ti = prepare.trace_inputs(prepare.diagram_project(p), path_indexes=(d.debug_ghost,))
    a = ti.args
    count = prepare.intersection_count(a.element_count)
    G = a.grid_count
    scale = np.float32(prepare.diagram_scale(p))
    try:
        cpu, kind, wl = orc.Reference(), 'reference', ti.wavelengths.astype(np.int32)
    except (OSError, RuntimeError):
        cpu, kind, wl = orc.Oracle('f32'), 'port', ti.wavelengths
    t0 = time.perf_counter()
    _, inter = cpu.trace_intersections(ti.elements, ti.paths, wl, a, count)
    part = inter.reshape(a.path_count, 1, G, G, count, 8)[:, :, :, (G - 1) // 2 + d.column_offset]
    want = cpu.diagram(ti.elements, a.aperture_index, scale, part[0, 0] if part.size else None,
                       d.resolution.width(), d.resolution.height())
    cpu_ms = (time.perf_counter() - t0) * 1e3
    return {
        'element': 'DIAGRAM', 'image': f'{d.resolution.width()}x{d.resolution.height()}', 'grid': G,
        'ghost_paths': a.path_count, 'gpu_ms': gpu_ms, 'cpu_ms': cpu_ms, 'cpu_kind': kind,
        'cpu_cores': os.cpu_count(), 'equal_to_cpu': bool(np.array_equal(got, want)),
    }


def run_e2e(w, args) -> dict:
    """Frames through Engine.render (FLARE_STARBURST) with host inputs and host output."""
    import numpy as np
    import torch

    from realflare_gb300 import prepare
    from realflare_gb300.data import RenderElement
    from realflare_gb300.engine import Engine

    p = w.project
    p.output.element = RenderElement.FLARE_STARBURST
    engine = Engine(cache=False)
    for _ in range(2):
        assert engine.render(p)
        engine.image.array
    times = []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ok = engine.render(p)
        img = engine.image.array  # device -> host
        times.append(time.perf_counter() - t0)
        assert ok and img.shape[-1] == 4
    ti = prepare.trace_inputs(p)
    sr = p.render.starburst.resolution
    h2d = ti.elements.nbytes + ti.paths.nbytes + ti.wavelengths.nbytes + sr.width() * sr.height() * 4
    d2h = int(np.prod(img.shape)) * 4 + 8
    return {'value': 1.0 / statistics.median(times), 'unit': 'frames/s', 'h2d_bytes_per_step': int(h2d),
            'd2h_bytes_per_step': int(d2h)}


if __name__ == '__main__':
    main()
