"""Image types and device marshalling.

``image`` is pyraft's host image: a numpy ndarray subclass carrying the
corners of its field of view (pyraft/raftypes.py:254-406), with the same
constructor arguments, defaults and attributes, so code written against
pyraft keeps working.  ``gpu_image`` is its device-resident counterpart: a
float32 CUDA tensor with the same corner attributes.  Every operator in this
package accepts either; host images are copied to the GPU, computed there,
and returned as host float64 ``image`` objects (as pyraft returns), while
``gpu_image`` inputs stay on the device.
"""
from __future__ import annotations

import numpy

from . import _native


class image(numpy.ndarray):
    """A sampled function on a rectangle: top_left = (x, y) of element
    [0, 0], bottom_right = (x, y) of element [-1, -1]; rows run along y.
    Arguments as pyraft.image: shape (tuple, ndarray or image), and either
    top_left/bottom_right or extent=(x0, x1, y0, y1) / x_extent / y_extent."""

    def __new__(subtype, shape, top_left=None, bottom_right=None, extent=None,
                x_extent=None, y_extent=None, **kwargs):
        has_extent = bool(extent or x_extent or y_extent)
        has_corner = bool(top_left or bottom_right)
        if has_extent and has_corner:
            raise TypeError('Mutually exclusive arguments given.')
        if has_extent:
            if extent:
                x_extent = (extent[0], extent[1])
                y_extent = (extent[2], extent[3])
            else:
                x_extent = x_extent or (-1.0, 1.0)
                y_extent = y_extent or (-1.0, 1.0)
            top_left = (x_extent[0], y_extent[1])
            bottom_right = (x_extent[1], y_extent[0])

        if isinstance(shape, image):
            if not has_extent:
                top_left = top_left or shape.top_left
                bottom_right = bottom_right or shape.bottom_right
            if kwargs:
                raise TypeError('Unhandled arguments!')
            obj = numpy.ndarray.__new__(subtype, shape.shape, dtype=shape.dtype)
            obj[...] = shape[...]
        else:
            if not has_extent:
                top_left = top_left or (-1.0, 1.0)
                bottom_right = bottom_right or (1.0, -1.0)
            if isinstance(shape, numpy.ndarray):
                if kwargs:
                    raise TypeError('Unhandled arguments!')
                obj = numpy.ndarray.__new__(subtype, shape.shape, dtype=shape.dtype)
                obj[...] = shape[...]
            else:
                kwargs.setdefault('dtype', numpy.float64)
                obj = numpy.ndarray.__new__(subtype, shape, **kwargs)
                obj[...] = 0.0

        if len(obj.shape) != len(top_left) or len(top_left) != len(bottom_right):
            raise TypeError('Dimensions must match!')
        obj.top_left = tuple(top_left)
        obj.bottom_right = tuple(bottom_right)
        obj.sampling_distances = _sampling(obj.shape, obj.top_left, obj.bottom_right)
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        self.top_left = getattr(obj, 'top_left', None)
        self.bottom_right = getattr(obj, 'bottom_right', None)
        self.sampling_distances = getattr(obj, 'sampling_distances', None)

    def __reduce__(self):
        state = list(numpy.ndarray.__reduce__(self))
        state[2] = (state[2], (self.top_left, self.bottom_right, self.sampling_distances))
        return tuple(state)

    def __setstate__(self, state):
        numpy.ndarray.__setstate__(self, state[0])
        self.top_left, self.bottom_right, self.sampling_distances = state[1]

    def sample_coordinates(self, idx):
        return (self.top_left[0] + idx[1] * self.sampling_distances[0],
                self.top_left[1] + idx[0] * self.sampling_distances[1])

    def get_y_coordinate(self, idx):
        return self.top_left[1] + idx * self.sampling_distances[1]

    def get_x_coordinate(self, idx):
        return self.top_left[0] + idx * self.sampling_distances[0]

    def extent(self):
        return (self.top_left[0], self.bottom_right[0], self.bottom_right[1], self.top_left[1])

    def cuda(self, device=None):
        """Copy to the GPU as a float32 gpu_image with the same corners."""
        import torch
        t = torch.from_numpy(numpy.ascontiguousarray(self, dtype=numpy.float32))
        return gpu_image(t.to(device or 'cuda'), self.top_left, self.bottom_right)


def _sampling(shape, tl, br):
    try:
        return ((br[0] - tl[0]) / (shape[1] - 1.0), (br[1] - tl[1]) / (shape[0] - 1.0))
    except (ZeroDivisionError, IndexError):
        return (0.0, 0.0)


class gpu_image:
    """Device-resident image or sinogram: ``data`` is a 2-D float32 CUDA
    tensor (any strides), ``top_left``/``bottom_right`` as in ``image``."""

    __slots__ = ('data', 'top_left', 'bottom_right')

    def __init__(self, data, top_left=(-1.0, 1.0), bottom_right=(1.0, -1.0)):
        import torch
        if not isinstance(data, torch.Tensor) or data.dim() != 2:
            raise TypeError('gpu_image wraps a 2-D torch tensor')
        if data.dtype != torch.float32 or not data.is_cuda:
            raise TypeError('gpu_image data must be a float32 CUDA tensor')
        self.data = data
        self.top_left = tuple(float(v) for v in top_left)
        self.bottom_right = tuple(float(v) for v in bottom_right)

    @property
    def shape(self):
        return tuple(self.data.shape)

    @property
    def sampling_distances(self):
        return _sampling(self.shape, self.top_left, self.bottom_right)

    def extent(self):
        return (self.top_left[0], self.bottom_right[0], self.bottom_right[1], self.top_left[1])

    def cpu(self):
        """Copy back as a float64 host ``image``."""
        arr = self.data.detach().cpu().numpy().astype(numpy.float64)
        return image(arr, top_left=self.top_left, bottom_right=self.bottom_right)

    def numpy(self):
        return self.data.detach().cpu().numpy()

    def __repr__(self):
        return (f'gpu_image(shape={self.shape}, top_left={self.top_left}, '
                f'bottom_right={self.bottom_right})')


# ----------------------------------------------------------------------------
# Marshalling

def corners_of(x, default_tl=(-1.0, 1.0), default_br=(1.0, -1.0)):
    tl = getattr(x, 'top_left', None) or default_tl
    br = getattr(x, 'bottom_right', None) or default_br
    return tuple(tl), tuple(br)


def to_gpu(x, default_tl=(-1.0, 1.0), default_br=(1.0, -1.0)):
    """Return (gpu_image, was_host) for an image, gpu_image, ndarray or
    CUDA tensor."""
    import torch
    if isinstance(x, gpu_image):
        return x, False
    if isinstance(x, torch.Tensor):
        if not x.is_cuda:
            raise TypeError('torch tensors must be on a CUDA device')
        tl, br = corners_of(x, default_tl, default_br)
        return gpu_image(x.float() if x.dtype != torch.float32 else x, tl, br), False
    tl, br = corners_of(x, default_tl, default_br)
    arr = numpy.ascontiguousarray(numpy.asarray(x), dtype=numpy.float32)
    return gpu_image(torch.from_numpy(arr).cuda(), tl, br), True


def rg_image(g: gpu_image) -> _native.RG_IMAGE:
    """rg_image view of a gpu_image: element (i, j) at
    data[i * column_stride + j * line_stride] (raft/raft_matrix.h:67-68)."""
    t = g.data
    return _native.RG_IMAGE(t.data_ptr(), t.shape[0], t.stride(1), t.shape[1], t.stride(0),
                            g.top_left[0], g.top_left[1], g.bottom_right[0], g.bottom_right[1])


def stream_ptr():
    import torch
    return torch.cuda.current_stream().cuda_stream


def workspace(nbytes: int):
    """Scratch for one call from torch's caching allocator (stream-ordered on
    the current stream), returned as (tensor, pointer)."""
    import torch
    if nbytes == 0:
        return None, None
    t = torch.empty(int(nbytes), dtype=torch.uint8, device='cuda')
    return t, t.data_ptr()


def new_gpu(shape, tl, br):
    import torch
    return gpu_image(torch.zeros(tuple(shape), dtype=torch.float32, device='cuda'), tl, br)


def finish(g: gpu_image, was_host: bool):
    return g.cpu() if was_host else g
