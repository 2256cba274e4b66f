"""Device memory and stream plumbing (torch), plus the Buffer/Image objects of the task API.

``Buffer``/``Image`` keep the meaning of the reference's lazy host/device mirrors
(``realflare/api/tasks/opencl.py:64-207``): ``.args`` identifies the inputs that produced
the object (the reference's lru_cache keys hash them), ``.array`` is the host numpy view,
fetched from the device on first access. Here the device side is a torch CUDA tensor that
stays resident between tasks.
"""
from __future__ import annotations

import typing

import numpy as np
import torch

from .data import RealflareError


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RealflareError('no CUDA device: the render path runs on the GPU only')
    return torch.device('cuda', torch.cuda.current_device())


def stream_handle(stream: torch.cuda.Stream | None = None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else int(t.data_ptr())


def empty(shape, dtype=torch.float32) -> torch.Tensor:
    return torch.empty(shape, dtype=dtype, device=require_cuda())


def to_device(array: np.ndarray, dtype=None) -> torch.Tensor:
    t = torch.from_numpy(np.ascontiguousarray(array))
    if dtype is not None:
        t = t.to(dtype)
    return t.to(require_cuda(), non_blocking=False)


class MemoryObject:
    def __init__(self, tensor: torch.Tensor | None = None, array: np.ndarray | None = None,
                 args: typing.Any = None) -> None:
        self._tensor = tensor
        self._array = array
        self._args = args
        self._hash = None

    def __hash__(self) -> int:
        if self._hash is None:
            self._hash = hash(self._args)
        return self._hash

    @property
    def args(self) -> typing.Any:
        return self._args

    @args.setter
    def args(self, value: typing.Any) -> None:
        self._hash = None
        self._args = value

    @property
    def tensor(self) -> torch.Tensor:
        if self._tensor is None:
            self._tensor = to_device(self._array)
        return self._tensor

    @property
    def array(self) -> np.ndarray:
        if self._array is None:
            t = self._tensor.detach()
            if t.is_cuda:
                # straight into page-locked memory (torch's caching host allocator keeps
                # the block for the next read): a 67 MB image in about 0.4 ms instead of
                # the pageable path's staging copy and memcpy (about 4.5 ms)
                host = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                host.copy_(t)
                self._array = host.numpy()
            else:
                self._array = t.numpy()
        return self._array

    def clear_array(self) -> None:
        self._array = None


class Image(MemoryObject):
    """A float32 image: (h, w) single channel or (h, w, 4) RGBA."""

    @property
    def shape(self) -> tuple:
        return tuple(self._tensor.shape if self._tensor is not None else self._array.shape)


class Rays(MemoryObject):
    """Traced rays: ``tensor`` is float32 [6, P * W * G^2] (pos.xy, pos_apt.xy, rrel,
    reflectance planes); ``shape`` is the reference's (paths, wavelengths, rays)."""

    def __init__(self, tensor: torch.Tensor, shape: tuple, args: typing.Any = None) -> None:
        super().__init__(tensor=tensor, args=args)
        self.shape = shape

    def to_reference_layout(self) -> np.ndarray:
        """The rays as the reference's ``ray_dtype`` records (pos.z and dir are zero)."""
        from .constants import ray_dtype

        planes = self.array
        out = np.zeros(self.shape, ray_dtype).reshape(-1)
        out['pos'][:, 0] = planes[0]
        out['pos'][:, 1] = planes[1]
        out['pos_apt'][:, 0] = planes[2]
        out['pos_apt'][:, 1] = planes[3]
        out['rrel'] = planes[4]
        out['reflectance'] = planes[5]
        return out.reshape(self.shape)
