"""Correlation plugin with the upstream per-window contract, computed on the GPU.

``CorrelGB300`` follows ``CorrelFFTNumpy`` (calcul/correl.py:665-685) and the
methods it inherits from ``CorrelFFTBase`` / ``CorrelBase``
(calcul/correl.py:167-281, 513-568):

* ``__call__(im0, im1) -> (correl, norm)``: float32 plane in the
  ``_like_fftshift`` layout (so that ``dx = ix0 - ix``) and a Python float with
  ``correl / norm`` in [-1, 1];
* ``compute_displacements_from_correl(correl, norm) -> (dx, dy, correl_max,
  other_peaks)``, raising ``PIVError`` (``explanation``, ``results``) like
  upstream, including the second-chance search that writes NaNs into the
  caller's plane when ``displacement_max`` is None, and the other peaks when
  ``nb_peaks_to_search > 1``;
* ``apply_subpix(dx, dy, correl)`` (any ``SubPix`` method: '2d_gaussian2' with its
  centroid fallback, '2d_gaussian', 'centroid', 'no_subpix');
* ``get_indices_no_displacement()``, ``displacement_max``.

Every computation runs in the CUDA library; the plugin only moves arrays.  It
registers as ``correlation_classes["gb300"]``, and :func:`register_upstream`
adds it to an installed fluidimage's registry so that
``params.piv0.method_correl = "gb300"`` selects it there.  For whole passes, use
``fluidimage_gb300.WorkPIV`` (one launch per pass instead of one per window).
"""

from __future__ import annotations

import numpy as np

from . import _lib as L
from .engine import SUPPORTED_WINDOWS, displacement_mask, parse_displacement_max
from .errors import ERROR_STRINGS, PIVError


def _dev():
    import torch

    return torch.device("cuda")


class CorrelGB300:
    """FFT cross-correlation of one window pair (or a batch) on the GPU."""

    _tag = "gb300"
    #: class of the errors the per-window methods raise; ``register_upstream`` makes
    #: it a subclass of the installed fluidimage's PIVError as well, so that
    #: upstream's ``except PIVError`` (works/piv/singlepass.py:328, 339;
    #: works/piv/fix.py:202) catches it
    _piv_error = PIVError

    def __init__(self, im0_shape, im1_shape=None, method_subpix="2d_gaussian2", nsubpix=None,
                 displacement_max=None, particle_radius=3, nb_peaks_to_search=1, mode=None):
        self.mode = mode
        if im1_shape is None:
            im1_shape = im0_shape
        im0_shape = tuple(int(n) for n in im0_shape)
        im1_shape = tuple(int(n) for n in im1_shape)
        if im0_shape != im1_shape:
            raise ValueError(
                "with this correlation method the input images have to have the same shape."
            )
        if im0_shape[0] != im0_shape[1] or im0_shape[0] not in SUPPORTED_WINDOWS:
            raise NotImplementedError(f"window {im0_shape} not supported: square {SUPPORTED_WINDOWS}")
        if method_subpix == "2d_gaussian2" and nsubpix is not None and nsubpix != 1:
            raise ValueError(
                "Subpixel method '2d_gaussian2' doesn't require nsubpix. "
                "In this case, nsubpix has to be equal to None."
            )
        if method_subpix not in L.SUBPIX_METHODS:
            raise ValueError(f"method has to be in {list(L.SUBPIX_METHODS)}")
        self.nsubpix = 1 if nsubpix is None else int(nsubpix)
        if not 1 <= self.nsubpix <= L.MAX_NSUBPIX:
            raise NotImplementedError(f"nsubpix must be in 1..{L.MAX_NSUBPIX} on this backend")
        if not 1 <= int(nb_peaks_to_search) <= L.MAX_PEAKS:
            raise NotImplementedError(f"nb_peaks_to_search must be in 1..{L.MAX_PEAKS}")
        self.method_subpix = method_subpix
        self._method = L.SUBPIX_METHODS[method_subpix]
        self._minv = None
        self.im0_shape = im0_shape
        self.im1_shape = im1_shape
        self.n = im0_shape[0]
        self.iy0, self.ix0 = (i // 2 - 1 for i in im0_shape)
        self.displacement_max = parse_displacement_max(displacement_max, im0_shape)
        self.particle_radius = particle_radius
        self.nb_peaks_to_search = nb_peaks_to_search
        mask, box = displacement_mask(self.n, self.displacement_max)
        self.where_large_displacement = mask
        self.start_stop_for_search0 = (box[0], box[1])
        self.start_stop_for_search1 = (box[2], box[3])
        self._box = box
        self._mask_dev = None

    # ---------------------------------------------------------------- geometry
    def compute_displacement_from_indices(self, ix, iy):
        return self.ix0 - ix, self.iy0 - iy

    def compute_indices_from_displacement(self, dx, dy):
        return self.ix0 - dx, self.iy0 - dy

    def get_indices_no_displacement(self):
        return self.iy0, self.ix0

    # ---------------------------------------------------------------- planes
    def correl_batch(self, ims0, ims1):
        """Planes and norms of a stack of window pairs ``(count, n, n)``."""
        import torch

        lib = L.load()
        w0 = torch.as_tensor(np.ascontiguousarray(ims0, dtype=np.float32), device=_dev())
        w1 = torch.as_tensor(np.ascontiguousarray(ims1, dtype=np.float32), device=_dev())
        if w0.dim() == 2:
            w0, w1 = w0[None], w1[None]
        count = w0.shape[0]
        if tuple(w0.shape[1:]) != self.im0_shape or w0.shape != w1.shape:
            raise ValueError("Bad im_crop shape.")
        planes = torch.empty_like(w0)
        norms = torch.empty(count, dtype=torch.float64, device=w0.device)
        L.check(lib.fi_correl_windows(L.ptr(w0), L.ptr(w1), count, self.n, L.ptr(planes),
                                      L.ptr(norms), L.stream_handle()), "fi_correl_windows")
        return planes.cpu().numpy(), norms.cpu().numpy()

    def __call__(self, im0, im1):
        """Correlation plane and norm of one window pair (correl.py:671-685)."""
        planes, norms = self.correl_batch(im0, im1)
        return planes[0], float(norms[0])

    # ---------------------------------------------------------------- peaks
    def _mask_device(self):
        import torch

        if self.where_large_displacement is not None and self._mask_dev is None:
            self._mask_dev = torch.as_tensor(self.where_large_displacement.astype(np.uint8),
                                             device=_dev())
        return self._mask_dev

    def _minv_device(self):
        import torch

        from .engine import subpix_pinv

        if self.method_subpix == "2d_gaussian" and self._minv is None:
            self._minv = torch.as_tensor(subpix_pinv(self.nsubpix), device=_dev())
        return self._minv

    def peaks_batch(self, planes, norms, apply_subpix=False):
        """Peak search (+ subpixel) of a stack of planes; returns per-plane arrays
        ``(dx, dy, correl_max, err, i0, i1, other_peaks)``; ``planes`` receives the
        second-chance NaN boxes like upstream (no displacement_max only).
        ``other_peaks`` is None (nb_peaks_to_search == 1) or per plane None (search
        raised) or a list of ``(dx, dy, correl_max)``."""
        import torch

        lib = L.load()
        p = torch.as_tensor(np.ascontiguousarray(planes, dtype=np.float32), device=_dev())
        if p.dim() == 2:
            p = p[None]
        count = p.shape[0]
        nrm = torch.as_tensor(np.asarray(norms, dtype=np.float64).reshape(-1), device=_dev())
        f32 = dict(dtype=torch.float32, device=p.device)
        dx, dy, cm = (torch.empty(count, **f32) for _ in range(3))
        err = torch.empty(count, dtype=torch.uint8, device=p.device)
        i0 = torch.empty(count, dtype=torch.int32, device=p.device)
        i1 = torch.empty(count, dtype=torch.int32, device=p.device)
        b = self._box
        nb = int(self.nb_peaks_to_search)
        K = nb - 1
        pc = pk = pe = None
        if K > 0:
            pc = torch.empty(count, dtype=torch.int32, device=p.device)
            pk = torch.empty(count * K * L.PEAK_FIELDS, **f32)
            pe = torch.empty(count * K, dtype=torch.uint8, device=p.device)
        L.check(lib.fi_peaks_from_planes(
            L.ptr(p), L.ptr(nrm), count, self.n, L.ptr(self._mask_device()), b[0], b[1], b[2],
            b[3], int(self.particle_radius), int(apply_subpix), self._method, self.nsubpix,
            L.ptr(self._minv_device()), nb, L.ptr(dx), L.ptr(dy), L.ptr(cm), L.ptr(err),
            L.ptr(i0), L.ptr(i1), L.ptr(pc), L.ptr(pk), L.ptr(pe), L.stream_handle()),
            "fi_peaks_from_planes")
        if isinstance(planes, np.ndarray) and self.where_large_displacement is None:
            planes[...] = p.cpu().numpy().reshape(planes.shape)
        other = None
        if K > 0:
            counts = pc.cpu().numpy()
            peaks = pk.view(count, K, L.PEAK_FIELDS).cpu().numpy()
            other = [None if counts[k] < 0 else
                     [(int(peaks[k, j, 0]), int(peaks[k, j, 1]), peaks[k, j, 2])
                      for j in range(int(counts[k]))] for k in range(count)]
        return (dx.cpu().numpy(), dy.cpu().numpy(), cm.cpu().numpy(), err.cpu().numpy(),
                i0.cpu().numpy(), i1.cpu().numpy(), other)

    def compute_displacements_from_correl(self, correl, norm=1.0):
        """(dx, dy, correl_max, other_peaks) of one plane (correl.py:226-275, 561-568)."""
        dx, dy, cm, err, i0, i1, other = self.peaks_batch(correl, [norm])
        cmax = 0.0 if norm == 0 else cm[0]
        e = int(err[0])
        if e == 5:
            raise AssertionError("correlation plane without finite value")
        if e:
            error = self._piv_error(explanation=ERROR_STRINGS[e])
            error.results = (int(dx[0]), int(dy[0]), cmax)
            raise error
        return int(dx[0]), int(dy[0]), cmax, (None if other is None else other[0])

    def apply_subpix(self, dx, dy, correl):
        """Subpixel displacement with the plugin's method (correl.py:277-281,
        subpix.py:107-218)."""
        import torch

        lib = L.load()
        ix, iy = self.compute_indices_from_displacement(dx, dy)
        p = torch.as_tensor(np.ascontiguousarray(correl, dtype=np.float32), device=_dev())
        ii0 = torch.tensor([int(iy)], dtype=torch.int32, device=p.device)
        ii1 = torch.tensor([int(ix)], dtype=torch.int32, device=p.device)
        ox = torch.empty(1, dtype=torch.float32, device=p.device)
        oy = torch.empty(1, dtype=torch.float32, device=p.device)
        err = torch.empty(1, dtype=torch.uint8, device=p.device)
        L.check(lib.fi_subpix_at(L.ptr(p), 1, self.n, L.ptr(ii0), L.ptr(ii1), self._method,
                                 self.nsubpix, L.ptr(self._minv_device()), L.ptr(ox), L.ptr(oy),
                                 L.ptr(err), L.stream_handle()), "fi_subpix_at")
        e = int(err.item())
        if e:
            raise self._piv_error(explanation=ERROR_STRINGS[e], result_compute_subpix=(iy, ix))
        return float(ox.item()), float(oy.item())


correlation_classes = {CorrelGB300._tag: CorrelGB300}


def register_upstream():
    """Add ``CorrelGB300`` to an installed fluidimage's ``correlation_classes``.

    Upstream's ``singlepass`` module imports the same dict object
    (works/piv/singlepass.py:24), so ``params.piv0.method_correl = "gb300"``
    then selects this plugin.  Returns False when fluidimage is not importable.
    """
    try:
        from fluidimage.calcul import correl as upstream
        from fluidimage.calcul.errors import PIVError as UpstreamPIVError
    except Exception:
        return False

    class _PIVError(PIVError, UpstreamPIVError):
        """A PIVError of both packages (upstream's handlers catch their own class)."""

        def __init__(self, *args, **kwargs):
            Exception.__init__(self, *args)
            self.explanation = "General no peak error"
            self.__dict__.update(kwargs)

    CorrelGB300._piv_error = _PIVError
    upstream.correlation_classes[CorrelGB300._tag] = CorrelGB300
    return True
