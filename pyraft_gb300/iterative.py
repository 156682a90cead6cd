"""EM and OSEM (pyraft/iterative/em.py:109-320).

* ``make_em(sino, shape, projection_method, backprojection_method)`` returns
  a one-iteration callable, ``em(sino, shape, niter)`` runs MLEM from x0 = 1
  with pyraft's defaults (DDA pair; default shape = nviews x nviews, as
  pyraft/iterative/em.py:153-154).
* ``em_gpu(s, img_size, niter)``: slant-stack MLEM (raft_em_gpu's role) with
  the matched adjoint as backprojector (true MLEM).
* ``osem(sino, shape, niter, nblocks)``: OSEM over interleaved view subsets
  of the slant-stack pair (pyraft's osem uses Fourier-slice operators over
  contiguous blocks, which need pynfft; see em.cu).
Guards everywhere: y / 0 -> 0, and pixels with zero sensitivity -> 0
(pyraft divides by zero there).  Every loop runs inside the library
(rg_em): no host round trip per iteration.
"""
from __future__ import annotations

import numpy

from . import _native
from .raftypes import finish, gpu_image, image, new_gpu, rg_image, stream_ptr, to_gpu, workspace
from .sinogram import method_id, radon_method


def _run_em(sino, x0, method, niter, nsubsets):
    """x0: gpu_image updated in place."""
    L = _native.load()
    a, b = rg_image(sino), rg_image(x0)
    ws_t, ws = workspace(L.rg_em_workspace(a, b, method, nsubsets))
    _native.check(L.rg_em(a, b, method, int(niter), int(nsubsets), ws,
                          ws_t.numel() if ws_t is not None else 0, stream_ptr()))


def _method(projection_method, backprojection_method, reference=False):
    """Native EM method id.  reference=True (slant-stack only) backprojects
    with the slant-stack backprojection instead of the matched adjoint, the
    pairing of the reference's GPU EM (raft/raft_em_gpu.cu:20-87)."""
    p, b = method_id(projection_method), method_id(backprojection_method)
    if p != b:
        raise TypeError('projection and backprojection methods must form a transpose pair '
                        '(both BRESENHAM or both SLANTSTACK)')
    if p == method_id(radon_method.BRESENHAM):
        if reference:
            raise TypeError('reference=True applies to the SLANTSTACK method')
        return _native.RG_BRESENHAM
    if p == method_id(radon_method.SLANTSTACK):
        return _native.RG_SLANTSTACK_BP if reference else _native.RG_SLANTSTACK
    raise TypeError('Unsupported method for EM!')


def _start(shape, kwargs):
    if isinstance(shape, (image, gpu_image)):
        if kwargs:
            raise TypeError('Unhandled arguments!')
        x, host = to_gpu(shape)
        x = gpu_image(x.data.clone(), x.top_left, x.bottom_right)
        return x, host
    probe = image((2, 2), **kwargs)
    x = new_gpu(shape, probe.top_left, probe.bottom_right)
    x.data.fill_(1.0)
    return x, None


def _finish_em(x, shape_host, sino_host):
    """Host result if the start image was a host image, or (for a shape
    tuple) if the sinogram was; device result otherwise."""
    return finish(x, sino_host if shape_host is None else shape_host)


def make_em(sino, shape, projection_method=radon_method.BRESENHAM,
            backprojection_method=radon_method.BRESENHAM, weight=None, reference=False,
            **kwargs):
    """One-iteration EM map x -> x * A^T(y / A x) / A^T 1 (reference=True:
    the slant-stack backprojection B in place of A^T)."""
    if weight is not None:
        raise TypeError('a precomputed weight is not supported; the sensitivity is computed '
                        'on the device in FP64')
    m = _method(projection_method, backprojection_method, reference)
    gs, _ = to_gpu(sino, (0.0, 1.0), (numpy.pi, -1.0))

    def em_step(x):
        gx, host = to_gpu(x)
        gx = gpu_image(gx.data.clone(), gx.top_left, gx.bottom_right)
        _run_em(gs, gx, m, 1, 1)
        return finish(gx, host)
    return em_step


def em(sino, shape=None, niter=5, method=radon_method.BRESENHAM, reference=False, **kwargs):
    """EM (pyraft/iterative/em.py:151-169).  reference=True with SLANTSTACK:
    backproject with the slant-stack backprojection, as the reference's GPU
    EM does, instead of the matched adjoint."""
    if shape is None:
        shape = [sino.shape[1], sino.shape[1]]
    x, host = _start(shape, kwargs)
    gs, shost = to_gpu(sino, (0.0, 1.0), (numpy.pi, -1.0))
    _run_em(gs, x, _method(method, method, reference), niter, 1)
    return _finish_em(x, host, shost)


def osem(sino, shape=None, niter=5, nblocks=4, method=radon_method.SLANTSTACK, reference=False,
         **kwargs):
    if shape is None:
        shape = [sino.shape[0], sino.shape[0]]
    x, host = _start(shape, kwargs)
    gs, shost = to_gpu(sino, (0.0, 1.0), (numpy.pi, -1.0))
    _run_em(gs, x, _method(method, method, reference), niter, nblocks)
    return _finish_em(x, host, shost)


_STATE_KEYS = ("niter", "nsubsets", "method", "shape", "image_corners", "sinogram")


def _state_mismatch(state, params):
    """Name of the first run parameter in which a saved state differs from
    this call's (None when they all match)."""
    for k in _STATE_KEYS:
        a, b = state.get(k), params.get(k)
        if isinstance(a, (list, tuple)) and isinstance(b, (list, tuple)):
            if len(a) != len(b) or any(abs(float(u) - float(v)) > 1e-12 * max(1.0, abs(float(v)))
                                       for u, v in zip(a, b)):
                return k
        elif a != b:
            return k
    return None


def _sinogram_fingerprint(gs):
    """Shape, corners, and the FP64 sum and sum of squares of a device
    sinogram: enough to tell a resumed run that it was given other data."""
    import torch
    d = gs.data.to(torch.float64)
    return [float(gs.shape[0]), float(gs.shape[1]), *map(float, gs.top_left),
            *map(float, gs.bottom_right), float(d.sum()), float((d * d).sum())]


def em_checkpointed(sino, shape=None, niter=5, nsubsets=1, method=radon_method.SLANTSTACK,
                    reference=False, checkpoint=None, every=1, max_subiterations=None,
                    **kwargs):
    """EM (nsubsets = 1) or OSEM over interleaved subsets that can be stopped
    and resumed at any sub-iteration.

    After every `every` sub-iterations the state -- the iterate, the number
    of sub-iterations done and the run's parameters (niter, nsubsets,
    method, shape, image corners and a fingerprint of the sinogram) -- is
    written to `checkpoint` with torch.save (to a temporary file first, then
    renamed, so an interrupted write leaves the previous state).  A call
    that finds `checkpoint` continues from it; a state saved for other
    parameters or another sinogram raises ValueError.  max_subiterations
    stops this call after that many sub-iterations (the run resumes on the
    next call).  Each call runs its sub-iterations through
    rg_em_subiterations, so a run split over calls reaches the iterate of an
    uninterrupted rg_em call (OSEM subsets up to the rounding order of the
    tile-driven Radon's atomic ray sums).

    Returns (x, state): x as em/osem return it, state the dict saved last
    (with "done" True once all niter * nsubsets sub-iterations have run)."""
    import os
    import torch
    if checkpoint is None:
        raise TypeError('em_checkpointed needs a checkpoint path')
    if every < 1:
        raise ValueError('every must be >= 1')
    if shape is None:
        shape = [sino.shape[0], sino.shape[0]]
    m = _method(method, method, reference)
    gs, shost = to_gpu(sino, (0.0, 1.0), (numpy.pi, -1.0))
    x, host = _start(shape, kwargs)
    params = {"niter": int(niter), "nsubsets": int(nsubsets), "method": int(m),
              "shape": [int(v) for v in x.shape], "image_corners": [*x.top_left, *x.bottom_right],
              "sinogram": _sinogram_fingerprint(gs)}
    total = int(niter) * int(nsubsets)
    done = 0
    if os.path.exists(checkpoint):
        state = torch.load(checkpoint, map_location="cpu", weights_only=True)
        bad = _state_mismatch(state, params)
        if bad is not None:
            raise ValueError(f'checkpoint {checkpoint} was saved for another run ({bad} differs)')
        x.data.copy_(state["x"].to(x.data.device))
        done = int(state["subiteration"])
    L = _native.load()
    a, b = rg_image(gs), rg_image(x)
    ws_t, ws = workspace(L.rg_em_workspace(a, b, m, int(nsubsets)))
    wsb = ws_t.numel() if ws_t is not None else 0
    budget = total - done if max_subiterations is None else min(total - done, max_subiterations)
    state = dict(params, subiteration=done, done=done >= total, x=x.data.cpu())
    while budget > 0:
        c = min(every, budget)
        _native.check(L.rg_em_subiterations(a, b, m, int(nsubsets), done, c, ws, wsb,
                                            stream_ptr()))
        done += c
        budget -= c
        state = dict(params, subiteration=done, done=done >= total, x=x.data.cpu())
        tmp = f"{checkpoint}.tmp"
        torch.save(state, tmp)
        os.replace(tmp, checkpoint)
    return _finish_em(x, host, shost), state


def em_gpu(*args):
    """pyraft's em_gpu(s, img_size=rays, niter=20): host sinogram on the
    default geometry -> (img_size, img_size) float32 array, with the
    reference GPU EM's operator pair (slant-stack Radon, slant-stack
    backprojection; raft/raft_em_gpu.cu:20-87)."""
    if len(args) == 0:
        raise TypeError('Not enough arguments!')
    s = args[0]
    n = args[1] if len(args) > 1 else s.shape[0]
    niter = args[2] if len(args) > 2 else 20
    src = image(numpy.asarray(s, dtype=numpy.float64), top_left=(0.0, 1.0),
                bottom_right=(numpy.pi, -1.0))
    out = em(src, (n, n), niter, method=radon_method.SLANTSTACK, reference=True)
    return numpy.asarray(out, dtype=numpy.float32)


def osem_batch(sinos, shapes=None, niter=5, nsubsets=10, graph=True, x0=None):
    """OSEM of many independent slices of uneven size in one batched call.

    sinos: list of (nrays_k, nviews_k) sinograms (image or gpu_image, corners
    as for osem).  shapes: list of (N_k, N_k) (default nrays_k) or None.
    x0: optional list of start images (default ones).  Every sub-iteration is
    three persistent launches over all slices; with graph=True one iteration
    is captured into a CUDA graph and replayed niter times.  Returns a list
    of results of the same kinds as the inputs."""
    import ctypes
    import torch
    L = _native.load()
    gs, hosts, xs = [], [], []
    for k, s in enumerate(sinos):
        g, host = to_gpu(s, (0.0, 1.0), (numpy.pi, -1.0))
        gs.append(g)
        hosts.append(host)
        n = (shapes[k][0] if shapes is not None else g.shape[0])
        if x0 is not None:
            xg, _ = to_gpu(x0[k])
            xs.append(gpu_image(xg.data.clone(), xg.top_left, xg.bottom_right))
        else:
            x = new_gpu((n, n), (-1.0, 1.0), (1.0, -1.0))
            x.data.fill_(1.0)
            xs.append(x)
    n = len(gs)
    S = (_native.RG_IMAGE * max(n, 1))(*[rg_image(g) for g in gs])
    I = (_native.RG_IMAGE * max(n, 1))(*[rg_image(x) for x in xs])
    ws_t, ws = workspace(L.rg_osem_batch_workspace(S, I, n, nsubsets))
    _native.check(L.rg_osem_batch(S, I, n, int(niter), int(nsubsets), 1 if graph else 0, ws,
                                  ws_t.numel() if ws_t is not None else 0, stream_ptr()))
    return [finish(x, h) for x, h in zip(xs, hosts)]


def em_plain(sino, size=None, niter=5, nsubsets=1):
    """The plain one-slice-per-call GPU form (rg_em_plain_host): host
    sinogram on the default geometry -> (size, size) float32 array."""
    s = numpy.ascontiguousarray(numpy.asarray(sino), dtype=numpy.float32)
    n = size or s.shape[0]
    out = numpy.zeros((n, n), dtype=numpy.float32)
    _native.check(_native.load().rg_em_plain_host(
        out.ctypes.data, s.ctypes.data, n, s.shape[0], s.shape[1], int(niter), int(nsubsets)))
    return out


def em_transmission_gpu(*args):
    """pyraft's em_transmission_gpu(s, f, d, img_size=rays, niter=20):
    transmission EM from raw counts s, flat field f and dark field d (host
    (rays, views) arrays on the default geometry) -> (img_size, img_size)
    float64 array.  The update is applied once per iteration (the reference
    applies it twice, raft/raft_transmission_em.cu:57,59)."""
    if len(args) < 3:
        raise TypeError('Not enough arguments!')
    s, f, d = args[0], args[1], args[2]
    n = args[3] if len(args) > 3 else s.shape[0]
    niter = args[4] if len(args) > 4 else 20
    corners = ((0.0, 1.0), (numpy.pi, -1.0))
    gs, _ = to_gpu(image(numpy.asarray(s, numpy.float64), top_left=corners[0],
                         bottom_right=corners[1]))
    gf, _ = to_gpu(image(numpy.asarray(f, numpy.float64), top_left=corners[0],
                         bottom_right=corners[1]))
    gd = None if d is None else to_gpu(image(numpy.asarray(d, numpy.float64),
                                             top_left=corners[0], bottom_right=corners[1]))[0]
    x = new_gpu((n, n), (-1.0, 1.0), (1.0, -1.0))
    x.data.fill_(1.0)
    L = _native.load()
    S, F, X = rg_image(gs), rg_image(gf), rg_image(x)
    D = rg_image(gd) if gd is not None else _native.RG_IMAGE(None, 0, 0, 0, 0, 0., 0., 0., 0.)
    ws_t, ws = workspace(L.rg_em_transmission_workspace(S, X))
    _native.check(L.rg_em_transmission(S, F, D, X, int(niter), ws,
                                       ws_t.numel() if ws_t is not None else 0, stream_ptr()))
    return numpy.asarray(x.cpu(), dtype=numpy.float64)
