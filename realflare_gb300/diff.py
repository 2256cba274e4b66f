"""Differentiable flare rendering: the gradient of an image loss with respect to the lens
surfaces' curvature radii, the axial gaps between them, their coating thicknesses and the
light position. No reference counterpart (the reference renders only).

``LensParameters`` maps the free parameters to the trace's per-element inputs with torch
operations (so torch differentiates the mapping): element ``center = sum of the previous
elements' distances + radius``, the stop halving the gap it sits in, and the light direction
``(x * sensor_w / 2, y * h / w * sensor_w / 2, focal_length)``. ``FlareFunction`` (a
``torch.autograd.Function``) renders the flare with the CUDA kernels and, in backward, runs
their adjoints: ``rf_raster_backward`` (a gather over the forward's tile lists),
``rf_vertex_backward``, ``rf_quad_setup_backward`` (the 1/quad-area intensity term) and
``rf_trace_adjoint`` (rays re-traced from their entry point, surfaces recomputed).

What the gradient includes: ray positions through the quad-area intensity and through the
aperture positions (ghost texture lookup) and rrel, the Fresnel/coating reflectance, and the
light direction through all of these. What it leaves out, by construction: coverage. Which
pixels a quad covers and its mean-value weights depend on the vertex positions only through
integer sample coordinates (the reference truncates them), so they are piecewise constant;
the change of covered pixels as quad edges move, including a ghost sliding across the
screen, is not part of the gradient. The gradient is the derivative of the rendered image
wherever no coverage changes.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import prepare
from ._abi import check, lib
from .data import Project, RealflareError
from .device import empty, require_cuda


@dataclass
class LensLayout:
    """Element-level structure of a lens model: which elements are free surfaces, where the
    stop sits, and the constants of the mapping."""
    surfaces: list          # element indices of the spherical surfaces (the stop excluded)
    stop: int               # element index of the stop
    back_distance: float    # distance of the last surface to the sensor (held fixed)
    base_distances: np.ndarray  # element distances of the model
    focal_length: float
    sensor_w: float
    aspect: float           # image height / width


def layout(project: Project) -> LensLayout:
    lens = project.flare.lens
    model = lens.lens_model
    if model is None:
        raise RealflareError('differentiation needs a lens model object')
    n = len(model.lens_elements)
    surfaces = [i for i in range(n) if i != model.aperture_index]
    dist = np.array([e.distance for e in model.lens_elements], np.float64)
    r = project.render.resolution
    return LensLayout(surfaces, model.aperture_index, float(dist[-1]), dist, float(model.focal_length),
                      float(lens.sensor_size.width()), r.height() / r.width())


class LensParameters:
    """The free parameters of a lens and light: ``radii`` (one per surface), ``gaps`` (axial
    distance from each surface to the next; a stop inside a gap sits at its middle),
    ``thickness`` (single-layer coating thickness in nm per surface) and ``light`` (the
    normalised field position)."""

    def __init__(self, project: Project, device=None) -> None:
        self.project = project
        self.layout = layout(project)
        lo = self.layout
        model = project.flare.lens.lens_model
        dev = device if device is not None else require_cuda()
        el = model.lens_elements
        radii = [el[i].radius for i in lo.surfaces]
        gaps = []
        for k in range(len(lo.surfaces) - 1):
            a, b = lo.surfaces[k], lo.surfaces[k + 1]
            gaps.append(float(sum(lo.base_distances[a:b])))
        thick = project.flare.lens.coating_thickness
        t = [float(thick[i]) if i < len(thick) and np.ndim(thick[i]) == 0 else 0.0 for i in lo.surfaces]
        pos = project.flare.light.position
        kw = dict(dtype=torch.float64, device=dev)
        self.radii = torch.tensor(radii, **kw)
        self.gaps = torch.tensor(gaps, **kw)
        self.thickness = torch.tensor(t, **kw)
        self.light = torch.tensor([pos.x(), pos.y()], **kw)

    def tensors(self) -> list:
        return [self.radii, self.gaps, self.thickness, self.light]

    def elements(self, radii, gaps, thickness, light, n_elements: int):
        """(radius, center, thickness, direction.xyz) per element as torch tensors.

        The map is affine in the parameters, so it is evaluated as one matrix-vector product
        (and torch differentiates it as one): the matrix and offset come from
        ``elements_direct`` (the map's definition) at the zero and unit parameter vectors,
        once per element count, device and dtype."""
        M, b = self._affine(n_elements, radii.device, radii.dtype)
        out = torch.addmv(b, M, torch.cat([radii, gaps, thickness, light]))
        n = n_elements
        return out[:n], out[n:2 * n], out[2 * n:3 * n], out[3 * n:3 * n + 3]

    def _affine(self, n_elements: int, device, dtype):
        key = (n_elements, str(device), dtype)
        cache = self.__dict__.setdefault('_affine_cache', {})
        if key not in cache:
            sizes = [self.radii.numel(), self.gaps.numel(), self.thickness.numel(), 2]

            def f(vec):
                r, g, t, l = torch.split(vec, sizes)
                return torch.cat(self.elements_direct(r, g, t, l, n_elements))

            zero = torch.zeros(sum(sizes), dtype=torch.float64)
            b = f(zero)
            M = torch.stack([f(e) - b for e in torch.eye(sum(sizes), dtype=torch.float64)], dim=1)
            cache[key] = (M.to(device=device, dtype=dtype), b.to(device=device, dtype=dtype))
        return cache[key]

    def elements_direct(self, radii, gaps, thickness, light, n_elements: int):
        """The map itself, op by op: (radius, center, thickness, direction.xyz)."""
        lo = self.layout
        dev, dt = radii.device, radii.dtype
        radius = torch.zeros(n_elements, device=dev, dtype=dt)
        radius = radius.index_put((torch.tensor(lo.surfaces, device=dev),), radii)
        # element distances: surface k's distance is its gap (half of it before the stop,
        # the stop taking the other half); the last surface keeps its back distance
        distances = []
        for k, s in enumerate(lo.surfaces):
            if k == len(lo.surfaces) - 1:
                distances.append(torch.tensor(lo.back_distance, device=dev, dtype=dt))
            elif lo.surfaces[k + 1] == s + 1:
                distances.append(gaps[k])
            else:  # the stop sits between s and the next surface
                distances.append(gaps[k] / 2)
                distances.append(gaps[k] / 2)
        distances.append(torch.tensor(0.0, device=dev, dtype=dt))  # the sensor
        d = torch.stack(distances)
        offset = torch.cat([torch.zeros(1, device=dev, dtype=dt), torch.cumsum(d, 0)[:-1]])
        center = offset + radius
        t = torch.zeros(n_elements, device=dev, dtype=dt)
        t = t.index_put((torch.tensor(lo.surfaces, device=dev),), thickness)
        direction = torch.stack([light[0] * lo.sensor_w / 2, light[1] * lo.aspect * lo.sensor_w / 2,
                                 torch.tensor(lo.focal_length, device=dev, dtype=dt)])
        return radius, center, t, direction


class DifferentiableRenderer:
    """The flare of one project (lens, ghosts, wavelengths, grid, image) as a differentiable
    function of ``LensParameters``. ``render(params)`` returns the (h, w, 4) image tensor.

    ``accurate=True`` runs the forward trace with the double-precision ray geometry
    (``rf_trace_accurate``): the image, its coverage and the vertex attributes the gradient
    is taken at are then those of the double evaluation of the trace, not the reference's
    FP32 values (the adjoint's re-trace stays FP32: it only evaluates the Jacobians)."""

    def __init__(self, project: Project, ghost: torch.Tensor, paths=None, stream=None,
                 accurate: bool = False) -> None:
        from .tasks import RasterizingTask

        require_cuda()
        self.lib = lib()
        self.project = project
        self.ghost = ghost
        self.inputs = prepare.trace_inputs(project, paths)
        if self.inputs is None:
            raise RealflareError('the lens has fewer than two elements')
        ti = self.inputs
        self.E = ti.args.element_count
        if np.any(ti.elements['coating_layers'][[i for i in range(self.E - 1)]] == 2):
            raise RealflareError('differentiation supports single-layer coatings')
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        dev = require_cuda()
        self.base_elements = torch.from_numpy(ti.elements.view(np.float32).reshape(self.E, 16).copy()).to(dev)
        self.paths = torch.from_numpy(ti.paths).to(dev)
        self.wavelengths = torch.from_numpy(ti.wavelengths).to(dev)
        a = ti.args
        self.P, self.W, self.G = a.path_count, a.wavelength_count, a.grid_count
        self.n_rays = ti.ray_count
        self.area, self.min_area = prepare.quad_constants(project)
        # 16-pixel tiles: a 512^2 image has 1024 of them, enough CTAs to fill the GPU
        self.raster_args = prepare.raster_args(project, self.P, self.W, tuple(ghost.shape[:2]), tile_size=16)
        self.task = RasterizingTask(self.stream)
        self.rays = empty((6, max(self.n_rays, 1)))
        self.params = LensParameters(project, dev)
        self.accurate = accurate

    # -- kernels --------------------------------------------------------------------
    def _element_buffer(self, radius, center, thickness) -> torch.Tensor:
        el = self.base_elements.clone()
        el[:, 0] = radius.to(torch.float32)
        el[:, 3] = center.to(torch.float32)
        el[:, 6] = thickness.to(torch.float32)
        return el

    def _trace_args(self, direction):
        a = prepare.TraceArgs.from_buffer_copy(self.inputs.args)
        d = direction.detach().to(torch.float32).cpu().tolist()
        for k in range(3):
            a.direction[k] = d[k]
        return a

    def forward_kernels(self, radius, center, thickness, direction) -> torch.Tensor:
        s = int(self.stream.cuda_stream)
        self.el = self._element_buffer(radius, center, thickness)
        self.targs = self._trace_args(direction)
        trace = self.lib.rf_trace_accurate if self.accurate else self.lib.rf_trace
        check(trace(self.el.data_ptr(), self.paths.data_ptr(), self.wavelengths.data_ptr(),
                    ctypes.byref(self.targs), self.rays.data_ptr(), s), 'rf_trace')
        from .device import Rays

        rays = Rays(self.rays, (self.P, self.W, self.G ** 2))
        self.bounds, self.inten, self.vtx = self.task.setup(self.project, rays)
        self.offsets, self.entries = self.task.bin(self.raster_args, self.bounds, self.vtx)
        h, w = self.raster_args.height, self.raster_args.width
        self.image = empty((h, w, 4))
        check(self.lib.rf_raster(self.vtx.data_ptr(), self.offsets.data_ptr(), self.entries.data_ptr(),
                                 self.ghost.data_ptr(), self.task.spectrum().data_ptr(), ctypes.byref(self.raster_args),
                                 self.image.data_ptr(), s), 'rf_raster')
        return self.image

    def backward_kernels(self, grad_image: torch.Tensor):
        """(grad radius, grad center, grad thickness per element, grad normalised direction)."""
        s = int(self.stream.cuda_stream)
        gi = grad_image.to(torch.float32).contiguous()
        n_vtx = self.P * self.G ** 2 * self.W + 1
        g_vtx = empty((n_vtx * 8,))
        check(self.lib.rf_raster_backward(self.vtx.data_ptr(), self.offsets.data_ptr(), self.entries.data_ptr(),
                                          self.ghost.data_ptr(), self.task.spectrum().data_ptr(),
                                          ctypes.byref(self.raster_args), self.image.data_ptr(), gi.data_ptr(),
                                          g_vtx.data_ptr(), s), 'rf_raster_backward')
        g_rays = empty((6, max(self.n_rays, 1)))
        g_inten = empty((max(self.P * (self.G - 1) ** 2 * self.W, 1),))
        check(self.lib.rf_vertex_backward(self.rays.data_ptr(), self.inten.data_ptr(), self.P, self.W, self.G,
                                          g_vtx.data_ptr(), g_rays.data_ptr(), g_inten.data_ptr(), s),
              'rf_vertex_backward')
        check(self.lib.rf_quad_setup_backward(self.rays.data_ptr(), self.P, self.W, self.G, self.area, self.min_area,
                                              g_inten.data_ptr(), g_rays.data_ptr(), s), 'rf_quad_setup_backward')
        g_el = empty((self.E, 4))
        g_dir = empty((3,))
        check(self.lib.rf_trace_adjoint(self.el.data_ptr(), self.paths.data_ptr(), self.wavelengths.data_ptr(),
                                        ctypes.byref(self.targs), g_rays.data_ptr(), g_el.data_ptr(), g_dir.data_ptr(),
                                        s), 'rf_trace_adjoint')
        self.grad_rays = g_rays
        return g_el[:, 0], g_el[:, 1], g_el[:, 2], g_dir

    def trace_kernels(self, radius, center, thickness, direction):
        """The trace alone: (rays (6, n): positions, aperture positions, rrel, reflectance;
        the element buffer and trace arguments, which its adjoint needs)."""
        s = int(self.stream.cuda_stream)
        el = self._element_buffer(radius, center, thickness)
        targs = self._trace_args(direction)
        rays = empty((6, max(self.n_rays, 1)))
        trace = self.lib.rf_trace_accurate if self.accurate else self.lib.rf_trace
        check(trace(el.data_ptr(), self.paths.data_ptr(), self.wavelengths.data_ptr(), ctypes.byref(targs),
                    rays.data_ptr(), s), 'rf_trace')
        return rays, el, targs

    def trace_backward(self, el, targs, grad_rays: torch.Tensor):
        """rf_trace_adjoint of a trace: (grad radius, center, thickness, normalised direction)."""
        s = int(self.stream.cuda_stream)
        g = grad_rays.to(torch.float32).contiguous()
        g_el = empty((self.E, 4))
        g_dir = empty((3,))
        check(self.lib.rf_trace_adjoint(el.data_ptr(), self.paths.data_ptr(), self.wavelengths.data_ptr(),
                                        ctypes.byref(targs), g.data_ptr(), g_el.data_ptr(), g_dir.data_ptr(), s),
              'rf_trace_adjoint')
        return g_el[:, 0], g_el[:, 1], g_el[:, 2], g_dir

    # -- torch ----------------------------------------------------------------------
    def render(self, radii, gaps, thickness, light) -> torch.Tensor:
        radius, center, t, direction = self.params.elements(radii, gaps, thickness, light, self.E)
        return FlareFunction.apply(radius, center, t, direction, self)

    def trace(self, radii, gaps, thickness, light) -> torch.Tensor:
        """The traced rays (6, n) as a differentiable function of the parameters."""
        radius, center, t, direction = self.params.elements(radii, gaps, thickness, light, self.E)
        return TraceFunction.apply(radius, center, t, direction, self)

    def splat(self, rays: torch.Tensor, sigma: float, channels: bool = False) -> torch.Tensor:
        """A smooth stand-in for the flare's energy distribution (the coarse stage of the
        recovery): every traced ray's energy at its sensor position, splatted bilinearly
        into the image and blurred by a Gaussian of ``sigma`` pixels.

        The flare gives each quad the energy area_orig x the mean of its corners' ghost
        texture, housing falloff and coating reflectance (fragment_shader with the 1 / area
        intensity, rasterizing.cl:471-506); so a ray's weight here is that product (ghost
        texture at the aperture position, smoothstep(1, 0.95, rrel), reflectance) times its
        wavelength's colour, and the blurred splat approximates the blurred flare wherever the
        blur is wider than the quads. Unlike the flare, it is smooth in the ray positions.
        Returns (h, w) with the AP1 channels summed, or with ``channels`` the three channels
        (3, h, w); row 0 at the top like the flare image."""
        import torch.nn.functional as F

        ra = self.raster_args
        h, w = ra.height, ra.width
        P, W, R = self.P, self.W, self.G ** 2
        x = rays[0] * ra.screen_transform + w / 2  # vertex_shader's pixel mapping
        y = rays[1] * ra.screen_transform + h / 2
        valid = torch.isfinite(rays[5])
        gs = ra.ghost_scale
        grid = torch.stack([rays[2] / gs, rays[3] / gs], -1).view(1, 1, -1, 2)
        gi = F.grid_sample(self.ghost.view(1, 1, *self.ghost.shape[:2]), torch.nan_to_num(grid), mode='bilinear',
                           padding_mode='zeros', align_corners=False).view(-1)
        t = ((rays[4] - 1.0) / (0.95 - 1.0)).clamp(0.0, 1.0)
        ri = t * t * (3.0 - 2.0 * t)
        refl = torch.nan_to_num(rays[5]).clamp_min(0.0)
        colour = self._colour_weights()  # (W, 3)
        colour = colour if channels else colour.sum(1, keepdim=True)
        nc = colour.shape[1]
        colour = colour.t().reshape(nc, 1, W, 1).expand(nc, P, W, R).reshape(nc, -1)
        wgt = torch.where(valid, gi * ri * refl, torch.zeros_like(refl))[None] * colour  # (nc, n)
        xs, ys = torch.nan_to_num(x) - 0.5, torch.nan_to_num(y) - 0.5
        x0, y0 = torch.floor(xs), torch.floor(ys)
        fx, fy = xs - x0, ys - y0
        img = torch.zeros(nc, h * w, device=rays.device, dtype=rays.dtype)
        for dx, dy, k in ((0, 0, (1 - fx) * (1 - fy)), (1, 0, fx * (1 - fy)), (0, 1, (1 - fx) * fy), (1, 1, fx * fy)):
            xi, yi = x0.long() + dx, y0.long() + dy
            inside = valid & (xi >= 0) & (xi < w) & (yi >= 0) & (yi < h)
            idx = torch.where(inside, (h - 1 - yi) * w + xi, torch.zeros_like(xi))
            img = img.index_add(1, idx, torch.where(inside, k, torch.zeros_like(k))[None] * wgt)
        img = img.view(nc, h, w)
        if not channels:
            return gaussian_blur(img[0], sigma)
        return torch.stack([gaussian_blur(img[c], sigma) for c in range(nc)])

    def _colour_weights(self) -> torch.Tensor:
        """Per wavelength, the AP1 colour its records get (W, 3): the spectrum texel at
        position (w + 0.5) / W (rasterizing.cl:617-645, nearest texel); the last wavelength
        only ends the last pair and weighs 0; one wavelength adds the fragment to every XYZ
        channel (rasterizing.cl:648-650)."""
        cache = self.__dict__.get('_colour')
        if cache is None:
            from .constants import light_spectrum

            W = self.W
            spec = light_spectrum().astype(np.float64)[:, :3]
            c = np.zeros((W, 3))
            for k in range(max(W - 1, 1)):
                xyz = spec[min(int((k + 0.5) / W * spec.shape[0]), spec.shape[0] - 1)] if W > 1 else np.ones(3)
                c[k] = XYZ_TO_AP1 @ xyz
            cache = torch.tensor(c, dtype=torch.float32, device=self.base_elements.device)
            self._colour = cache
        return cache


# color.cl:3-10
XYZ_TO_AP1 = np.array([[1.6410233797, -0.3248032942, -0.2364246952],
                       [-0.6636628587, 1.6153315917, 0.0167563477],
                       [0.0117218943, -0.0082844420, 0.9883948585]])


def gaussian_blur(img: torch.Tensor, sigma: float) -> torch.Tensor:
    """Separable Gaussian blur (zero outside the image) of an (h, w) tensor."""
    import torch.nn.functional as F

    r = max(1, int(3 * sigma))
    k = torch.exp(-0.5 * (torch.arange(-r, r + 1, device=img.device, dtype=img.dtype) / sigma) ** 2)
    k = k / k.sum()
    x = F.conv2d(img[None, None], k.view(1, 1, 1, -1), padding=(0, r))
    x = F.conv2d(x, k.view(1, 1, -1, 1), padding=(r, 0))
    return x[0, 0]


def _direction_backward(direction: torch.Tensor, g_n: torch.Tensor) -> torch.Tensor:
    """n = normalize(-v), v = direction: dn/dv = -(I - n n^T) / |v|."""
    v = direction.to(torch.float64)
    norm = torch.linalg.norm(v)
    n = -v / norm
    g_n = g_n.to(torch.float64)
    return (-(g_n - n * torch.dot(n, g_n)) / norm).to(direction.dtype)


class TraceFunction(torch.autograd.Function):
    """rays = trace(radius, center, coating thickness per element, light direction.xyz); each
    call keeps its own element buffer and trace arguments for its adjoint, so several traces
    (other light positions) can precede one backward."""

    @staticmethod
    def forward(ctx, radius, center, thickness, direction, renderer: DifferentiableRenderer):
        ctx.renderer = renderer
        ctx.save_for_backward(direction)
        with torch.no_grad():
            rays, ctx.el, ctx.targs = renderer.trace_kernels(radius, center, thickness, direction)
        return rays

    @staticmethod
    def backward(ctx, grad_rays):
        (direction,) = ctx.saved_tensors
        g_radius, g_center, g_thick, g_n = ctx.renderer.trace_backward(ctx.el, ctx.targs, grad_rays)
        dt = direction.dtype
        return (g_radius.to(dt), g_center.to(dt), g_thick.to(dt), _direction_backward(direction, g_n), None)


class FlareFunction(torch.autograd.Function):
    """image = flare(radius, center, coating thickness per element, light direction.xyz)."""

    @staticmethod
    def forward(ctx, radius, center, thickness, direction, renderer: DifferentiableRenderer):
        ctx.renderer = renderer
        ctx.save_for_backward(direction)
        with torch.no_grad():
            image = renderer.forward_kernels(radius, center, thickness, direction)
        return image.clone()

    @staticmethod
    def backward(ctx, grad_image):
        (direction,) = ctx.saved_tensors
        r = ctx.renderer
        g_radius, g_center, g_thick, g_n = r.backward_kernels(grad_image)
        # n = normalize(-v), v = direction: dn/dv = -(I - n n^T) / |v|
        v = direction.to(torch.float64)
        norm = torch.linalg.norm(v)
        n = -v / norm
        g_n = g_n.to(torch.float64)
        g_v = -(g_n - n * torch.dot(n, g_n)) / norm
        dt = direction.dtype
        return (g_radius.to(dt), g_center.to(dt), g_thick.to(dt), g_v.to(dt), None)
