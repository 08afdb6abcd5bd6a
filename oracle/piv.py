"""numpy restatement of the upstream fluidimage 0.5.3 PIV path — TEST INFRASTRUCTURE ONLY.

Every function names the upstream file:line it restates (paths inside the
fluidimage project).  The arithmetic follows the upstream code as it runs when
its ``@boost`` functions execute as plain Python ("pure-Python transonic mode"),
which is how the golden vectors in ``tests/golden`` were recorded:

* FFTs are numpy pocketfft on float32 input, hence complex64 (numpy >= 2);
* peak search, second-chance search and the '2d_gaussian2' fit use float32
  arithmetic with the same operation order;
* WorkFIX neighbour means are float32; TPS is float64 with LAPACK ``gesv``.

``dtype_complex=np.complex128`` gives the FP64 variant used to state the GPU
error against an FP64 oracle.

Window-level work is vectorised over all windows of a pass (numpy), so that the
same module also serves as the CPU baseline ("port") timed by ``bench.py``.
"""

from __future__ import annotations

import math
from types import SimpleNamespace

import numpy as np

ERR_NONE = 0
ERR_BOUNDARY = 1
ERR_NAN = 2
ERR_WRONG_SUBPIX = 3
ERR_BAD_CROP = 4
ERR_ALL_NAN = 5
ERR_CLOSE_BOUNDARY = 6

ERROR_STRINGS = {
    ERR_BOUNDARY: "Correlation peak touching boundary.",
    ERR_NAN: "Correlation peak touching nan.",
    ERR_WRONG_SUBPIX: "wrong subpix",
    ERR_BAD_CROP: "Bad im_crop shape.",
    ERR_ALL_NAN: "Correlation plane without any finite value.",
    ERR_CLOSE_BOUNDARY: "close boundary",
}

_F32_1EM8 = np.float32(1e-8)


def _f32_pow2(a):
    """``x ** 2`` on float32 scalars as numpy evaluates it in the upstream source
    (subpix.py:57-58, :201): through the C library's ``powf``, which can round a
    near-tie the other way from ``x * x`` (4.2536864**2 lies 0.49994 ulp above a
    float32; ``powf`` returns the upper neighbour).  Element by element for that
    reason; the CUDA kernels use the correctly rounded product."""
    a = np.asarray(a, dtype=np.float32)
    return np.fromiter((v ** 2 for v in a.ravel()), dtype=np.float32,
                       count=a.size).reshape(a.shape)


# ----------------------------------------------------------------------------------
# a1: window grid — works/piv/singlepass.py:108-141 and _init_crop :363-389
# ----------------------------------------------------------------------------------
def crop_start_stop(shape_crop):
    """``_start_for_crop`` / ``_stop_for_crop`` (singlepass.py:363-389)."""
    n0, n1 = shape_crop
    start = (n0 // 2, n1 // 2)
    stop = (n0 // 2 + (n0 % 2), n1 // 2 + (n1 % 2))
    return start, stop


def make_grid(imshape, shape_crop, overlap):
    """``_prepare_with_image`` (singlepass.py:108-141): 1-D vectors ``ixvecs, iyvecs``."""
    len_y, len_x = imshape
    start, stop = crop_start_stop(shape_crop)
    stepy = shape_crop[0] - int(np.round(overlap * shape_crop[0]))
    stepx = shape_crop[1] - int(np.round(overlap * shape_crop[1]))
    assert stepy >= 1 and stepx >= 1
    ixvec_max = len_x - stop[1]
    ixvecs = np.arange(start[1], ixvec_max, stepx, dtype=int)
    iyvec_max = len_y - stop[0]
    iyvecs = np.arange(start[0], iyvec_max, stepy, dtype=int)
    if ixvec_max - ixvecs[-1] > stepx // 2.5:
        ixvecs = np.append(ixvecs, ixvec_max)
    if iyvec_max - iyvecs[-1] > stepy // 2.5:
        iyvecs = np.append(iyvecs, iyvec_max)
    return ixvecs, iyvecs


def grid_flat(ixvecs, iyvecs):
    """Row-major flatten of the meshgrid (singlepass.py:136-141)."""
    gx, gy = np.meshgrid(ixvecs, iyvecs)
    return gx.flatten(), gy.flatten()


# ----------------------------------------------------------------------------------
# a2: padding — singlepass.py:196-208
# ----------------------------------------------------------------------------------
def pad_images(im0, im1, shape_crop):
    start, stop = crop_start_stop(shape_crop)
    npad = max(start + stop)
    pads = [(npad, npad), (npad, npad)]
    im0pad = np.pad(im0 - im0.min(), pads, "constant", constant_values=0)
    im1pad = np.pad(im1 - im1.min(), pads, "constant", constant_values=0)
    return im0pad, im1pad, npad


# ----------------------------------------------------------------------------------
# a3: window positions — singlepass.py:210-260 (pass 0), :787-870 (pass >= 1)
# ----------------------------------------------------------------------------------
def positions_first_pass(ixvecs_grid, iyvecs_grid, npad):
    ix = ixvecs_grid + npad
    iy = iyvecs_grid + npad
    return ixvecs_grid, iyvecs_grid, ix, iy, ix, iy


def positions_from_displacement(ixvecs_grid, iyvecs_grid, dxin, dyin, imshape, npad):
    """``WorkPIVFromDisplacement._calcul_positions_vectors_subimages`` (:787-870)."""
    ixs0 = ixvecs_grid - dxin // 2
    iys0 = iyvecs_grid - dyin // 2
    ixs1 = ixs0 + dxin
    iys1 = iys0 + dyin
    ny, nx = imshape
    out1 = (ixs1 > nx) | (iys1 > ny) | (ixs1 < 0) | (iys1 < 0)
    out0 = (ixs0 > nx) | (iys0 > ny) | (ixs0 < 0) | (iys0 < 0)
    a = out1
    b = ~out1 & out0
    ixs0 = np.where(a, ixvecs_grid - dxin, np.where(b, ixvecs_grid, ixs0))
    iys0 = np.where(a, iyvecs_grid - dyin, np.where(b, iyvecs_grid, iys0))
    ixs1 = np.where(a, ixvecs_grid, np.where(b, ixvecs_grid + dxin, ixs1))
    iys1 = np.where(a, iyvecs_grid, np.where(b, iyvecs_grid + dyin, iys1))
    xs = (ixs0 + ixs1) / 2.0
    ys = (iys0 + iys1) / 2.0
    return xs, ys, ixs0 + npad, iys0 + npad, ixs1 + npad, iys1 + npad


# ----------------------------------------------------------------------------------
# a4: cropping — singlepass.py:391-407 (numpy slice semantics, incl. negative starts)
# ----------------------------------------------------------------------------------
def _slice_bounds(start, stop, length):
    """Effective ``[s, e)`` of ``arr[start:stop]`` on an axis of ``length`` (vectorised)."""
    start = np.asarray(start, dtype=np.int64)
    stop = np.asarray(stop, dtype=np.int64)
    s = np.where(start < 0, np.maximum(start + length, 0), np.minimum(start, length))
    e = np.where(stop < 0, np.maximum(stop + length, 0), np.minimum(stop, length))
    return s, np.maximum(e, s)


def crop_windows(impad, ixs_pad, iys_pad, shape_crop):
    """Stack of windows (float32) and a mask of windows with the right shape."""
    start, stop = crop_start_stop(shape_crop)
    n0, n1 = shape_crop
    Ly, Lx = impad.shape
    sy, ey = _slice_bounds(iys_pad - start[0], iys_pad + stop[0], Ly)
    sx, ex = _slice_bounds(ixs_pad - start[1], ixs_pad + stop[1], Lx)
    valid = ((ey - sy) == n0) & ((ex - sx) == n1)
    sy = np.where(valid, sy, 0)
    sx = np.where(valid, sx, 0)
    rows = sy[:, None] + np.arange(n0)[None, :]
    cols = sx[:, None] + np.arange(n1)[None, :]
    wins = impad[rows[:, :, None], cols[:, None, :]].astype(np.float32)
    return wins, valid


# ----------------------------------------------------------------------------------
# a5 / a7: FFT correlation — calcul/correl.py:671-685, calcul/fft.py:254-269,
#          _like_fftshift correl.py:596-636
# ----------------------------------------------------------------------------------
def like_fftshift(arr):
    """``fftshift(arr[::-1, ::-1])`` over the last two axes (correl.py:596-636)."""
    return np.ascontiguousarray(np.fft.fftshift(arr[..., ::-1, ::-1], axes=(-2, -1)))


def correl_fft(wins0, wins1, dtype_complex=np.complex64):
    """Batched ``CorrelFFTNumpy.__call__``: returns ``(planes, norms)``.

    ``norm = sqrt(4 E0 E1) * N`` with ``E = sum|F|^2 / 2 / N^2`` (fft.py:107-109,
    259-269); energies are summed in the FFT's real precision.
    """
    nvec, n0, n1 = wins0.shape
    N = n0 * n1
    real = np.float32 if dtype_complex == np.complex64 else np.float64
    w0 = wins0.astype(real, copy=False)
    w1 = wins1.astype(real, copy=False)
    F0 = np.fft.fft2(w0)
    F0[:, 0, 0] = 0.0
    F1 = np.fft.fft2(w1)
    F1[:, 0, 0] = 0.0
    correl = np.fft.ifft2(F0.conj() * F1).real
    e0 = np.empty(nvec, dtype=real)
    e1 = np.empty(nvec, dtype=real)
    a0 = abs(F0) ** 2
    a1 = abs(F1) ** 2
    for i in range(nvec):
        e0[i] = np.sum(a0[i]) / 2 / N**2
        e1[i] = np.sum(a1[i]) / 2 / N**2
    norms = np.array(
        [math.sqrt(4 * e0[i] * e1[i]) * N for i in range(nvec)], dtype=np.float64
    )
    planes = like_fftshift(np.ascontiguousarray(correl))
    return planes.astype(real, copy=False), norms


# ----------------------------------------------------------------------------------
# a8: displacement_max mask and search box — correl.py:68-73, 518-547
# ----------------------------------------------------------------------------------
def parse_displacement_max(displ_max, shape):
    if isinstance(displ_max, str) and displ_max.endswith("%"):
        return float(displ_max[:-1]) / 100 * max(shape)
    return displ_max


def indices_no_displacement(shape_crop):
    """``iy0, ix0 = n // 2 - 1`` (correl.py:189)."""
    return shape_crop[0] // 2 - 1, shape_crop[1] // 2 - 1


def displacement_mask(shape_crop, displacement_max):
    """Mask of ``|d| > displacement_max`` and the search box (correl.py:518-547)."""
    n0, n1 = shape_crop
    iy0, ix0 = indices_no_displacement(shape_crop)
    if displacement_max is None:
        return None, (0, n0), (0, n1)
    mask = np.zeros((n0, n1), dtype=bool)
    for i0 in range(n0):
        for i1 in range(n1):
            dx = ix0 - i1
            dy = iy0 - i0
            if math.sqrt(dx**2 + dy**2) > displacement_max:
                mask[i0, i1] = True
    for i0_start in range(n0):
        if not all(mask[i0_start, :]):
            break
    for i1_start in range(n1):
        if not all(mask[:, i1_start]):
            break
    for i0_stop in range(n0 - 1, -1, -1):
        if not all(mask[i0_stop, :]):
            break
    i0_stop += 1
    for i1_stop in range(n1 - 1, -1, -1):
        if not all(mask[:, i1_stop]):
            break
    i1_stop += 1
    return mask, (i0_start, i0_stop), (i1_start, i1_stop)


# ----------------------------------------------------------------------------------
# a9: peak search — nan_indices_max correl.py:88-132, _compute_indices_max :135-164
# ----------------------------------------------------------------------------------
def nan_indices_max(planes, box0, box1):
    """Vectorised ``nan_indices_max``: last maximum in row-major order wins (``>=``).

    Returns ``(i0, i1, err)`` with ``err`` in {0, ERR_BOUNDARY, ERR_NAN, ERR_ALL_NAN}.
    """
    nvec, n0, n1 = planes.shape
    flat = planes.reshape(nvec, n0 * n1)
    start_flat = box0[0] * n1 + box1[0]
    tail = flat[:, start_flat:]
    finite = ~np.isnan(tail)
    has_init = finite.any(axis=1)
    first = np.argmax(finite, axis=1)
    init = tail[np.arange(nvec), first]

    box = planes[:, box0[0] : box0[1], box1[0] : box1[1]]
    bn0 = box.shape[1]
    bn1 = box.shape[2]
    bflat = box.reshape(nvec, bn0 * bn1)
    bfinite = ~np.isnan(bflat)
    any_box = bfinite.any(axis=1)
    filled = np.where(bfinite, bflat, -np.inf)
    mbox = filled.max(axis=1)
    eq = (filled == mbox[:, None]) & bfinite
    last = bn0 * bn1 - 1 - np.argmax(eq[:, ::-1], axis=1)
    take_box = any_box & (mbox >= init)
    i0 = np.where(take_box, box0[0] + last // bn1, 0)
    i1 = np.where(take_box, box1[0] + last % bn1, 0)

    err = np.zeros(nvec, dtype=np.uint8)
    boundary = (i0 == 0) | (i0 == n0 - 1) | (i1 == 0) | (i1 == n1 - 1)
    err[boundary] = ERR_BOUNDARY
    inner = np.nonzero(~boundary)[0]
    if inner.size:
        r = i0[inner][:, None, None] + np.arange(-1, 2)[None, :, None]
        c = i1[inner][:, None, None] + np.arange(-1, 2)[None, None, :]
        nb = planes[inner[:, None, None], r, c]
        has_nan = np.isnan(nb).reshape(inner.size, 9).any(axis=1)
        err[inner[has_nan]] = ERR_NAN
    err[~has_init] = ERR_ALL_NAN
    return i0, i1, err


def _correl_max(planes, i0, i1, norms):
    """``correl[iy, ix] / norm`` in float32, 0.0 when ``norm == 0`` (correl.py:151-155)."""
    vals = planes[np.arange(planes.shape[0]), i0, i1]
    out = np.empty(planes.shape[0], dtype=np.float32)
    for k in range(planes.shape[0]):
        if norms[k] == 0:
            out[k] = 0.0
        else:
            out[k] = vals[k] / np.float32(norms[k])
    return out


# ----------------------------------------------------------------------------------
# a10: second-chance search — correl.py:226-275 and CorrelFFTBase :561-568
# ----------------------------------------------------------------------------------
def displacements_from_correl(planes, norms, shape_crop, displacement_max=None,
                              particle_radius=3, nb_peaks=1):
    """Batched ``compute_displacements_from_correl`` for the FFT correlation classes.

    ``planes`` is modified in place exactly like the upstream per-window call: when
    ``displacement_max`` is None the second-chance NaN box is written into the
    caller's plane.  Returns ``(dx, dy, correl_max, err, i0, i1)`` where ``err`` is
    the error of the final attempt (0 if the peak is valid) and ``dx, dy`` are
    integers.
    """
    nvec, n0, n1 = planes.shape
    iy0, ix0 = indices_no_displacement(shape_crop)
    mask, box0, box1 = displacement_mask(shape_crop, displacement_max)
    if mask is not None:
        work = planes.copy()
        work[:, mask] = np.nan
    else:
        work = planes
    i0, i1, err = nan_indices_max(work, box0, box1)
    cmax = _correl_max(work, i0, i1, norms)

    retry = np.nonzero((err != 0) & (err != ERR_ALL_NAN))[0]
    r = particle_radius
    for k in retry:
        sy, ey = _slice_bounds(i0[k] - r, i0[k] + r + 1, n0)
        sx, ex = _slice_bounds(i1[k] - r, i1[k] + r + 1, n1)
        work[k, int(sy):int(ey), int(sx):int(ex)] = np.nan
    if retry.size:
        j0, j1, err2 = nan_indices_max(work[retry], box0, box1)
        cmax2 = _correl_max(work[retry], j0, j1, norms[retry])
        ok = err2 == 0
        good = retry[ok]
        i0[good] = j0[ok]
        i1[good] = j1[ok]
        cmax[good] = cmax2[ok]
        err[retry] = err2
    dx = ix0 - i1
    dy = iy0 - i0
    if nb_peaks <= 1:
        return dx, dy, cmax, err, i0, i1
    other = secondary_peaks(work, norms, err, i0, i1, shape_crop, box0, box1, nb_peaks,
                            particle_radius)
    return dx, dy, cmax, err, i0, i1, other


def secondary_peaks(work, norms, err, i0, i1, shape_crop, box0, box1, nb_peaks,
                    particle_radius=3):
    """Other peaks of ``compute_displacements_from_correl`` (correl.py:250-273).

    For each window whose search did not raise, NaN boxes of ``particle_radius``
    around the last peak found (on a copy of the searched plane, which holds the
    displacement mask and the second-chance box) and a new search, up to
    ``nb_peaks - 1`` times, stopping at the first search that raises.  Returns a
    list with None for the windows whose search raised, else a list of
    ``(dx, dy, correl_max)`` (integers, float32).  A plane without any finite value
    left stops the search (upstream's assert in nan_indices_max).
    """
    nvec, n0, n1 = work.shape
    iy0, ix0 = indices_no_displacement(shape_crop)
    r = particle_radius
    out = [None] * nvec
    for k in range(nvec):
        if err[k] != 0:
            continue
        c = work[k].copy()
        a0, a1 = int(i0[k]), int(i1[k])
        peaks = []
        for _ in range(nb_peaks - 1):
            sy, ey = _slice_bounds(a0 - r, a0 + r + 1, n0)
            sx, ex = _slice_bounds(a1 - r, a1 + r + 1, n1)
            c[int(sy):int(ey), int(sx):int(ex)] = np.nan
            j0, j1, e = nan_indices_max(c[None], box0, box1)
            if e[0] != 0:
                break
            a0, a1 = int(j0[0]), int(j1[0])
            cm = _correl_max(c[None], j0, j1, norms[k:k + 1])[0]
            peaks.append((ix0 - a1, iy0 - a0, cm))
        out[k] = peaks
    return out


# ----------------------------------------------------------------------------------
# a11: subpixel fit — calcul/subpix.py:16-61 ('2d_gaussian2'), :107-218 (SubPix)
# ----------------------------------------------------------------------------------
def _gaussian2(crops):
    """'2d_gaussian2' on a stack of 3x3 crops (subpix.py:16-61): float32 like the
    upstream code for float32 planes, float64 throughout for float64 planes (the
    FP64 oracle)."""
    real = np.float64 if crops.dtype == np.float64 else np.float32
    pow2 = _f32_pow2 if real is np.float32 else (lambda a: a * a)
    c = crops.astype(real, copy=True)
    cmin = c.reshape(-1, 9).min(axis=1)
    c -= cmin[:, None, None]
    cmax = c.reshape(-1, 9).max(axis=1)
    with np.errstate(invalid="ignore", divide="ignore"):
        c /= cmax[:, None, None]
    c[c == 0] = real(1e-8)
    with np.errstate(invalid="ignore", divide="ignore"):
        L = np.log(c)
    z = np.zeros(c.shape[0], dtype=real)
    c10, c01, c11, c20, c02 = z.copy(), z.copy(), z.copy(), z.copy(), z.copy()
    with np.errstate(invalid="ignore", over="ignore"):
        for a in range(3):
            for b in range(3):
                l = L[:, a, b]
                c10 = c10 + real(b - 1) * l
                c01 = c01 + real(a - 1) * l
                c11 = c11 + real((b - 1) * (a - 1)) * l
                c20 = c20 + real(3 * (b - 1) ** 2 - 2) * l
                c02 = c02 + real(3 * (a - 1) ** 2 - 2) * l
        c10 = c10 / real(6)
        c01 = c01 / real(6)
        c11 = c11 / real(4)
        c20 = c20 / real(6)
        c02 = c02 / real(6)
        den = real(4) * c20 * c02 - pow2(c11)
        deplx = (c11 * c01 - real(2) * c10 * c02) / den
        deply = (c11 * c10 - real(2) * c01 * c20) / den
    return deplx, deply


_XC = np.array([[-1.0, 0.0, 1.0]] * 3)
_YC = _XC.T.copy()


def subpix_2d_gaussian2(planes, i0, i1, shape_crop):
    """``apply_subpix`` with method '2d_gaussian2' and its centroid fallback (float32
    arithmetic for float32 planes, float64 for the FP64 oracle's float64 planes).

    Returns ``(deltax, deltay, wrong)``; where ``wrong`` is True the upstream code
    raises ``PIVError('wrong subpix')`` and keeps the integer displacement.
    """
    nvec = planes.shape[0]
    iy0, ix0 = indices_no_displacement(shape_crop)
    idx = np.arange(nvec)
    r = i0[:, None, None] + np.arange(-1, 2)[None, :, None]
    c = i1[:, None, None] + np.arange(-1, 2)[None, None, :]
    crops = planes[idx[:, None, None], r, c]
    deplx, deply = _gaussian2(crops)
    real = deplx.dtype.type
    pow2 = _f32_pow2 if real is np.float32 else (lambda a: a * a)
    with np.errstate(invalid="ignore", over="ignore"):
        big = (pow2(deplx) + pow2(deply)) > real(4.5)
    dx = np.empty(nvec, dtype=real)
    dy = np.empty(nvec, dtype=real)
    wrong = np.zeros(nvec, dtype=bool)
    with np.errstate(invalid="ignore", over="ignore"):
        gx = real(ix0) - (deplx + i1.astype(real))
        gy = real(iy0) - (deply + i0.astype(real))
    dx[:] = gx
    dy[:] = gy
    for k in np.nonzero(big)[0]:
        crop = crops[k]
        s = np.sum(crop)
        cx = np.sum(_XC * crop) / s
        cy = np.sum(_YC * crop) / s
        if cx**2 + cy**2 > 4.5:
            wrong[k] = True
            dx[k] = ix0 - i1[k]
            dy[k] = iy0 - i0[k]
        else:
            dx[k] = ix0 - (cx + i1[k])
            dy[k] = iy0 - (cy + i0[k])
    return dx, dy, wrong


SUBPIX_METHODS = ("2d_gaussian", "2d_gaussian2", "centroid", "no_subpix")


def subpix_setup(nsubpix):
    """``SubPix.prepare_subpix`` (subpix.py:86-105): half width, centroid grids and the
    pseudo-inverse used by '2d_gaussian'."""
    n = 1 if nsubpix is None else int(nsubpix)
    xs = np.arange(-n, n + 1, dtype=float)
    X, Y = np.meshgrid(xs, xs)
    Xr, Yr = X.ravel(), Y.ravel()
    M = np.reshape(np.concatenate((Xr**2, Yr**2, Xr, Yr, np.ones(Xr.size))), (5, Xr.size)).T
    return n, X, Y, np.linalg.pinv(M)


def subpix_one(plane, i0, i1, shape_crop, method, nsubpix=None):
    """``apply_subpix`` / ``SubPix.compute_subpix`` on one plane (correl.py:277-281,
    subpix.py:107-218), any method.  Returns ``(dx, dy, err)``; on an error
    (ERR_WRONG_SUBPIX, ERR_CLOSE_BOUNDARY) the integer displacement."""
    n, X, Y, Minv = subpix_setup(nsubpix)
    iy0, ix0 = indices_no_displacement(shape_crop)
    ny, nx = plane.shape

    def run(meth):
        if i0 - n < 0 or i0 + n + 1 > ny or i1 - n < 0 or i1 + n + 1 > nx:
            return None, ERR_CLOSE_BOUNDARY
        with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
            if meth == "2d_gaussian":
                crop = plane[i0 - n:i0 + n + 1, i1 - n:i1 + n + 1]
                cmap = crop.ravel().copy()
                cmap[cmap <= 0.0] = 1e-6
                coef = np.dot(Minv, np.log(cmap))
                if coef[0] > 0 or coef[1] > 0:
                    return run("centroid")
                sigmax = 1 / np.sqrt(-2 * coef[0])
                sigmay = 1 / np.sqrt(-2 * coef[1])
                deplx = coef[2] * sigmax**2
                deply = coef[3] * sigmay**2
                if np.isnan(deplx) or np.isnan(deply):
                    return run("centroid")
            elif meth == "2d_gaussian2":
                gx, gy = _gaussian2(plane[None, i0 - 1:i0 + 2, i1 - 1:i1 + 2])
                deplx, deply = gx[0], gy[0]
            elif meth == "centroid":
                crop = plane[i0 - n:i0 + n + 1, i1 - n:i1 + n + 1]
                s = np.sum(crop)
                deplx = np.sum(X * crop) / s
                deply = np.sum(Y * crop) / s
            else:
                deplx = deply = 0.0
            if deplx**2 + deply**2 > 2 * (0.5 + n) ** 2:
                if meth == "2d_gaussian2":
                    return run("centroid")
                return None, ERR_WRONG_SUBPIX
        return (deplx + i1, deply + i0), 0

    res, err = run(method)
    if err:
        return float(ix0 - i1), float(iy0 - i0), err
    return ix0 - res[0], iy0 - res[1], 0


# ----------------------------------------------------------------------------------
# a12 / a15: one PIV pass — singlepass.py:262-361 and :733-785
# ----------------------------------------------------------------------------------
def piv_pass(im0, im1, shape_crop, overlap, *, grid=None, dxin=None, dyin=None,
             apply_subpix=True, displacement_max=None, particle_radius=3,
             dtype_complex=np.complex64, keep_planes=False, method_subpix="2d_gaussian2",
             nsubpix=None, nb_peaks_to_search=1):
    """One pass.  Returns a namespace with the ``HeavyPIVResults`` fields."""
    shape_crop = tuple(int(n) for n in shape_crop)
    if grid is None:
        grid = make_grid(im0.shape, shape_crop, overlap)
    ixvecs, iyvecs = grid
    gx, gy = grid_flat(ixvecs, iyvecs)
    im0pad, im1pad, npad = pad_images(im0, im1, shape_crop)
    if dxin is None:
        xs, ys, ix0p, iy0p, ix1p, iy1p = positions_first_pass(gx, gy, npad)
    else:
        xs, ys, ix0p, iy0p, ix1p, iy1p = positions_from_displacement(
            gx, gy, dxin, dyin, im0.shape, npad
        )
    w0, v0 = crop_windows(im0pad, ix0p, iy0p, shape_crop)
    w1, v1 = crop_windows(im1pad, ix1p, iy1p, shape_crop)
    valid = v0 & v1
    nvec = gx.size
    dmax = parse_displacement_max(displacement_max, shape_crop)

    # float32 results like upstream; float64 ones for the FP64 oracle
    real = np.float32 if dtype_complex == np.complex64 else np.float64
    deltaxs = np.full(nvec, np.nan, dtype=real)
    deltays = np.full(nvec, np.nan, dtype=real)
    correls_max = np.full(nvec, np.nan, dtype=np.float32)
    err = np.full(nvec, ERR_BAD_CROP, dtype=np.uint8)
    planes_all = None
    secondary = [None] * nvec

    iv = np.nonzero(valid)[0]
    if iv.size:
        planes, norms = correl_fft(w0[iv], w1[iv], dtype_complex)
        out = displacements_from_correl(
            planes, norms, shape_crop, dmax, particle_radius, nb_peaks_to_search
        )
        dx, dy, cmax, e, i0, i1 = out[:6]
        if nb_peaks_to_search > 1:
            for j, k in enumerate(iv):
                secondary[k] = out[6][j]
        fdx = dx.astype(real)
        fdy = dy.astype(real)
        ok = e == 0
        if apply_subpix and ok.any():
            k = np.nonzero(ok)[0]
            if method_subpix == "2d_gaussian2":
                sdx, sdy, wrong = subpix_2d_gaussian2(planes[k], i0[k], i1[k], shape_crop)
                fdx[k] = sdx
                fdy[k] = sdy
                e[k[wrong]] = ERR_WRONG_SUBPIX
            else:
                for kk in k:
                    a, b, ee = subpix_one(planes[kk], int(i0[kk]), int(i1[kk]), shape_crop,
                                          method_subpix, nsubpix)
                    fdx[kk] = a
                    fdy[kk] = b
                    e[kk] = ee
        deltaxs[iv] = fdx
        deltays[iv] = fdy
        correls_max[iv] = cmax
        err[iv] = e
        if keep_planes:
            planes_all = np.full((nvec,) + shape_crop, np.nan, dtype=planes.dtype)
            planes_all[iv] = planes
    if dxin is not None:
        deltaxs += dxin
        deltays += dyin

    errors = {int(i): ERROR_STRINGS[int(err[i])] for i in np.nonzero(err)[0]}
    return SimpleNamespace(
        deltaxs=deltaxs, deltays=deltays, xs=xs, ys=ys, correls_max=correls_max,
        errors=errors, err=err, ixvecs=ixvecs, iyvecs=iyvecs, ixvecs_grid=gx,
        iyvecs_grid=gy, planes=planes_all, shape_crop=shape_crop,
        deltaxs_input=dxin, deltays_input=dyin, secondary_peaks=secondary,
        nb_peaks_to_search=nb_peaks_to_search, method_subpix=method_subpix, nsubpix=nsubpix,
    )


# ----------------------------------------------------------------------------------
# a13: WorkFIX — works/piv/fix.py:66-133, calcul/mean_neighbors.py:5-155
# ----------------------------------------------------------------------------------
def mean_neighbors(arr, not_nan):
    """NaN-aware 8-neighbour mean in float32 (mean_neighbors.py:5-125).

    ``arr`` holds zeros where ``not_nan`` is False.  Summation order follows the
    upstream loops: the two horizontal neighbours first, then the column pairs.
    """
    a = arr.astype(np.float32)
    b = not_nan.astype(np.float32)
    n0, n1 = a.shape
    out = np.zeros_like(a)
    cnt = np.zeros_like(a)
    ap = np.zeros((n0 + 2, n1 + 2), np.float32)
    bp = np.zeros((n0 + 2, n1 + 2), np.float32)
    ap[1:-1, 1:-1] = a
    bp[1:-1, 1:-1] = b

    def sh(p, d0, d1):
        return p[1 + d0 : 1 + d0 + n0, 1 + d1 : 1 + d1 + n1]

    # core order: (left + right), then for idx in -1, 0, 1: (up[i1-idx] + down[i1-idx])
    core_a = sh(ap, 0, -1) + sh(ap, 0, 1)
    core_b = sh(bp, 0, -1) + sh(bp, 0, 1)
    for idx in (-1, 0, 1):
        core_a = core_a + (sh(ap, -1, -idx) + sh(ap, 1, -idx))
        core_b = core_b + (sh(bp, -1, -idx) + sh(bp, 1, -idx))
    out[1:-1, 1:-1] = core_a[1:-1, 1:-1]
    cnt[1:-1, 1:-1] = core_b[1:-1, 1:-1]

    # edges and corners follow their own upstream orders
    def edge_row(i0, dn):
        for i1 in range(1, n1 - 1):
            ta = a[i0, i1 - 1] + a[i0, i1 + 1]
            tb = b[i0, i1 - 1] + b[i0, i1 + 1]
            for idx in (-1, 0, 1):
                ta = ta + a[i0 + dn, i1 - idx]
                tb = tb + b[i0 + dn, i1 - idx]
            out[i0, i1] = ta
            cnt[i0, i1] = tb

    def edge_col(i1, dn):
        for i0 in range(1, n0 - 1):
            ta = a[i0 - 1, i1] + a[i0 + 1, i1]
            tb = b[i0 - 1, i1] + b[i0 + 1, i1]
            for idx in (-1, 0, 1):
                ta = ta + a[i0 + idx, i1 + dn]
                tb = tb + b[i0 + idx, i1 + dn]
            out[i0, i1] = ta
            cnt[i0, i1] = tb

    edge_row(0, 1)
    edge_row(n0 - 1, -1)
    edge_col(0, 1)
    edge_col(n1 - 1, -1)
    for (i0, i1, d0, d1) in ((0, 0, 1, 1), (0, n1 - 1, 1, -1), (n0 - 1, 0, -1, 1),
                             (n0 - 1, n1 - 1, -1, -1)):
        out[i0, i1] = (a[i0 + d0, i1] + a[i0 + d0, i1 + d1]) + a[i0, i1 + d1]
        cnt[i0, i1] = (b[i0 + d0, i1] + b[i0 + d0, i1 + d1]) + b[i0, i1 + d1]

    with np.errstate(invalid="ignore", divide="ignore"):
        res = out / cnt
    res[(~not_nan) | (cnt == 0)] = np.nan
    return res.astype(np.float32)


def mean_neighbors_xy(deltaxs, deltays, ny, nx):
    """``mean_neighbors_xy`` (mean_neighbors.py:128-155)."""
    dx = deltaxs.reshape(ny, nx).copy()
    dy = deltays.reshape(ny, nx).copy()
    bad = np.isnan(dx) | np.isnan(dy)
    dx[bad] = 0.0
    dy[bad] = 0.0
    return (mean_neighbors(dx, ~bad).reshape(-1), mean_neighbors(dy, ~bad).reshape(-1))


def fix(result, correl_min=0.2, threshold_diff_neighbour=10, displacement_max=None):
    """``WorkFIX.calcul`` (fix.py:66-243); in place.

    With ``result.nb_peaks_to_search >= 2`` the secondary peaks replace a vector when
    one lies closer to the neighbour mean (fix.py:135-236); this needs the planes
    (``result.planes``) for the subpixel fit of the chosen peak.
    """
    deltaxs = result.deltaxs
    deltays = result.deltays
    errors = result.errors
    wrong_x, wrong_y = {}, {}
    for ierr in list(errors.keys()):
        wrong_x[ierr] = deltaxs[ierr]
        wrong_y[ierr] = deltays[ierr]
        deltaxs[ierr] = np.nan
        deltays[ierr] = np.nan

    def put_to_nan(inds, explanation):
        for ind in inds:
            ind = int(ind)
            if ind not in wrong_x:
                wrong_x[ind] = deltaxs[ind]
                wrong_y[ind] = deltays[ind]
                deltaxs[ind] = np.nan
                deltays[ind] = np.nan
                errors[ind] = explanation
            else:
                errors[ind] += " + " + explanation

    inds = (result.correls_max < correl_min).nonzero()[0]
    put_to_nan(inds, "correl < correl_min")
    if displacement_max:
        with np.errstate(invalid="ignore"):
            inds = ((deltaxs**2 + deltays**2) > displacement_max**2).nonzero()[0]
        put_to_nan(inds, "delta2 < displacement_max2")
    d2 = mx = my = None
    if threshold_diff_neighbour is not None:
        ny, nx = len(result.iyvecs), len(result.ixvecs)
        mx, my = mean_neighbors_xy(deltaxs, deltays, ny, nx)
        with np.errstate(invalid="ignore"):
            d2 = (mx - deltaxs) ** 2 + (my - deltays) ** 2
            inds = (d2 > threshold_diff_neighbour**2).nonzero()[0]
        put_to_nan(inds, "diff neighbour too large")
        for ivec in inds:
            errors[ivec] += f" (diff = {math.sqrt(d2[ivec]):.2f})"
        result.deltaxs_wrong = wrong_x
        result.deltays_wrong = wrong_y
    if getattr(result, "nb_peaks_to_search", 1) < 2:
        return result
    # secondary peaks (fix.py:135-236)
    ratio = np.float32(0.6)
    cmin32 = np.float32(correl_min)
    replaced = {}
    for ivec, other in enumerate(result.secondary_peaks):
        if not other:
            continue
        correl0 = result.correls_max[ivec]
        if result.deltaxs_input is not None:
            dxi = int(result.deltaxs_input[ivec])
            dyi = int(result.deltays_input[ivec])
        else:
            dxi = dyi = 0
        good = []
        with np.errstate(invalid="ignore", divide="ignore"):
            for dx, dy, corr in other:
                if np.float32(corr) / correl0 > ratio and np.float32(corr) > cmin32:
                    good.append((int(dx) + dxi, int(dy) + dyi, np.float32(corr)))
        if not good:
            continue
        if d2 is None:
            raise NameError("name 'differences2' is not defined")
        dn = np.empty(len(good) + 1)
        dn[0] = math.sqrt(d2[ivec]) if not np.isnan(d2[ivec]) else np.nan
        for i, (dx, dy, corr) in enumerate(good):
            dn[i + 1] = np.sqrt((float(mx[ivec]) - dx) ** 2 + (float(my[ivec]) - dy) ** 2)
        am = int(np.argmin(dn))
        if am == 0:
            continue
        dx, dy, corr = good[am - 1]
        if threshold_diff_neighbour is not None and dn[am] > threshold_diff_neighbour:
            continue
        if displacement_max and dx**2 + dy**2 > displacement_max:
            continue
        iy0, ix0 = indices_no_displacement(result.shape_crop)
        # upstream's peak indices are Python ints on the first pass and int32 after
        # (deltaxs_input is an int32 array): the subpixel sums are then float64
        cast = int if result.deltaxs_input is None else np.int32
        sdx, sdy, e = subpix_one(result.planes[ivec], cast(iy0 - (dy - dyi)),
                                 cast(ix0 - (dx - dxi)), result.shape_crop,
                                 result.method_subpix, result.nsubpix)
        if e:
            continue
        ndx, ndy = sdx + dxi, sdy + dyi
        old = (wrong_x.get(ivec, deltaxs[ivec]), wrong_y.get(ivec, deltays[ivec]),
               result.correls_max[ivec])
        replaced[ivec] = old
        deltaxs[ivec] = ndx
        deltays[ivec] = ndy
        result.correls_max[ivec] = corr
        if ivec in errors:
            del wrong_x[ivec], wrong_y[ivec], errors[ivec]
    if replaced:
        result.replaced_vectors = replaced
    return result


# ----------------------------------------------------------------------------------
# a14: thin-plate spline — calcul/interpolate/thin_plate_spline.py:108-216,
#      thin_plate_spline_subdom.py:25-280
# ----------------------------------------------------------------------------------
def tps_matrix(new_pos, centers):
    """``compute_tps_matrix_numpy`` (thin_plate_spline.py:108-165): ``(N+3, M)``."""
    d, m = new_pos.shape
    _, n = centers.shape
    em = np.zeros((n, m))
    for ind_d in range(d):
        ds, cs = np.meshgrid(new_pos[ind_d], centers[ind_d])
        em += (ds - cs) ** 2
    nz = np.where(em != 0)
    em[nz] = em[nz] * np.log(em[nz]) / 2
    return np.vstack([em, np.ones(m), new_pos])


def tps_weights(centers, values, smoothing):
    """``compute_tps_weights`` (thin_plate_spline.py:168-216)."""
    nb_dim, n = centers.shape
    rhs = np.hstack([values, np.zeros(nb_dim + 1)]).reshape(-1, 1)
    em = tps_matrix(centers, centers).T
    sm = np.hstack([smoothing * np.eye(n, n), np.zeros([n, nb_dim + 1])])
    pm = np.hstack([np.ones([n, 1]), centers.T])
    im = np.vstack([em + sm, np.hstack([pm.T, np.zeros([nb_dim + 1, nb_dim + 1])])])
    w = np.linalg.solve(im, rhs)
    return np.dot(em, w).ravel(), w.ravel()


class TPSSubdom:
    """``ThinPlateSplineSubdom`` (thin_plate_spline_subdom.py:25-280)."""

    def __init__(self, centers, subdom_size, smoothing_coef, threshold=None,
                 percent_buffer_area=20):
        self.centers = centers
        self.threshold = threshold
        xs = centers[1]
        ys = centers[0]
        self.num_centers = xs.size
        x_min, x_max = xs.min(), xs.max()
        y_min, y_max = ys.min(), ys.max()
        range_x = x_max - x_min
        range_y = y_max - y_min
        aspect_ratio = range_y / range_x
        nb_subdom = xs.size / subdom_size
        nbx = int(np.floor(math.sqrt(nb_subdom / aspect_ratio))) or 1
        nby = int(np.ceil(math.sqrt(nb_subdom * aspect_ratio))) or 1
        self.nb_subdomx, self.nb_subdomy = nbx, nby
        self.nb_subdom = nbx * nby
        x_dom = np.linspace(x_min, x_max, nbx + 1)
        y_dom = np.linspace(y_min, y_max, nby + 1)
        per_subdom = xs.size / self.nb_subdom
        self.smoothing_coef = smoothing_coef * math.sqrt(
            (x_dom[1] - x_dom[0]) * (y_dom[1] - y_dom[0]) / per_subdom
        )
        coef = percent_buffer_area / 100
        bx = coef * range_x / nbx
        by = coef * range_y / nby
        self.lim_min_x = x_dom[:-1] - bx
        self.lim_max_x = x_dom[1:] + bx
        self.lim_min_y = y_dom[:-1] - by
        self.lim_max_y = y_dom[1:] + by
        self.xmax_d = np.empty(self.nb_subdom)
        self.ymax_d = np.empty(self.nb_subdom)
        self.xc_d = np.empty(self.nb_subdom)
        self.yc_d = np.empty(self.nb_subdom)
        self.indices = []
        i = 0
        for iy in range(nby):
            for ix in range(nbx):
                xmin, xmax = self.lim_min_x[ix], self.lim_max_x[ix]
                ymin, ymax = self.lim_min_y[iy], self.lim_max_y[iy]
                self.indices.append(
                    np.where((xs >= xmin) & (xs < xmax) & (ys >= ymin) & (ys < ymax))[0]
                )
                self.xmax_d[i] = xmax
                self.ymax_d[i] = ymax
                self.xc_d[i] = 0.5 * (xmin + xmax)
                self.yc_d[i] = 0.5 * (ymin + ymax)
                i += 1
        self.norm_coefs = np.zeros(self.num_centers)
        self.norm_coefs_d = []
        for i in range(self.nb_subdom):
            ind = self.indices[i]
            c = self._coef_norm(xs[ind], ys[ind], i)
            self.norm_coefs_d.append(c)
            self.norm_coefs[ind] += c

    def _coef_norm(self, xs, ys, i):
        dxm = self.xmax_d[i] - self.xc_d[i]
        dym = self.ymax_d[i] - self.yc_d[i]
        dx2 = (xs - self.xc_d[i]) ** 2 / dxm**2
        dy2 = (ys - self.yc_d[i]) ** 2 / dym**2
        return (1 - dx2) * (1 - dy2) + 0.001

    def weights_iter(self, centers, values):
        summary = {"nb_fixed_vectors": 0}
        smoothed, w = tps_weights(centers, values, self.smoothing_coef)
        count = 1
        if self.threshold is not None:
            diff = np.sqrt((smoothed - values) ** 2)
            bad = np.argwhere(diff > self.threshold)
            summary["max(Udiff)"] = max(diff)
            nfixed = 0
            while bad.size != 0:
                nfixed += bad.size
                values[bad] = smoothed[bad]
                smoothed, w = tps_weights(centers, values, self.smoothing_coef)
                diff = np.sqrt((smoothed - values) ** 2)
                bad = np.argwhere(diff > self.threshold)
                count += 1
                if count > 10:
                    break
            summary["nb_fixed_vectors"] = nfixed
        summary["nb_iterations"] = count
        return smoothed, w, summary

    def weights_subdom(self, values):
        smoothed_d, w_d, summaries = [], [], []
        for i in range(self.nb_subdom):
            s, w, summ = self.weights_iter(self.centers[:, self.indices[i]],
                                           values[self.indices[i]])
            smoothed_d.append(s)
            w_d.append(w)
            summaries.append(summ)
        smoothed = np.zeros(self.num_centers)
        for i in range(self.nb_subdom):
            smoothed[self.indices[i]] += self.norm_coefs_d[i] * smoothed_d[i]
        smoothed /= self.norm_coefs
        return smoothed, w_d, summaries

    def init_new_positions(self, new_pos):
        xs = new_pos[1]
        ys = new_pos[0]
        self.num_new = xs.size
        self.ind_new = []
        for iy in range(self.nb_subdomy):
            for ix in range(self.nb_subdomx):
                self.ind_new.append(np.where(
                    (xs >= self.lim_min_x[ix]) & (xs < self.lim_max_x[ix])
                    & (ys >= self.lim_min_y[iy]) & (ys < self.lim_max_y[iy]))[0])
        self.norm_new = np.zeros(self.num_new)
        self.norm_new_d = []
        for i in range(self.nb_subdom):
            ind = self.ind_new[i]
            c = self._coef_norm(xs[ind], ys[ind], i)
            self.norm_new_d.append(c)
            self.norm_new[ind] += c
        self.mats = [tps_matrix(new_pos[:, self.ind_new[i]],
                                self.centers[:, self.indices[i]])
                     for i in range(self.nb_subdom)]

    def interpolate(self, w_d):
        out = np.zeros(self.num_new)
        for i in range(self.nb_subdom):
            out[self.ind_new[i]] += self.norm_new_d[i] * np.dot(w_d[i], self.mats[i])
        out /= self.norm_new
        return out


class InterpError(ValueError):
    pass


def griddata(centers, values, xnew, ynew):
    """``calcul/interpolate/griddata.py:11-27``: linear, then nearest where NaN."""
    from scipy import interpolate

    gx, gy = np.meshgrid(xnew, ynew)
    out = interpolate.griddata(centers.T, values, (gx, gy), "linear")
    inds = np.where(np.isnan(out))
    nearest = interpolate.griddata(centers.T, values, (gx, gy), "nearest")
    out[inds] = nearest[inds]
    return out.flatten()


def apply_interp(result, grid_next, params_mp, last=False):
    """``BaseWorkPIV.apply_interp`` (singlepass.py:409-563).

    ``grid_next`` = ``(ixvecs, iyvecs)`` (1-D) of the work doing the interpolation.
    Sets ``deltaxs_approx`` (or ``_final``, ``_smooth``) on ``result``.
    """
    ixvecs, iyvecs = grid_next
    gx, gy = grid_flat(ixvecs, iyvecs)
    if last:
        result.ixvecs_final, result.iyvecs_final = gx, gy
    else:
        result.ixvecs_approx, result.iyvecs_approx = gx, gy
    sel = ~(np.isnan(result.deltaxs) | np.isnan(result.deltays))
    if not sel.any():
        raise InterpError("Only nan.")
    xs = result.xs[sel]
    ys = result.ys[sel]
    centers = np.vstack([ys, xs])
    dxs = result.deltaxs[sel]
    dys = result.deltays[sel]
    use_tps = params_mp.use_tps is True or (params_mp.use_tps == "last" and last)
    if use_tps:
        tps = TPSSubdom(centers, params_mp.subdom_size, params_mp.smoothing_coef,
                        threshold=params_mp.threshold_tps, percent_buffer_area=20)
        try:
            sx, wx, summ_x = tps.weights_subdom(dxs)
            sy, wy, summ_y = tps.weights_subdom(dys)
        except np.linalg.LinAlgError:
            use_tps = False
        else:
            tps.init_new_positions(np.vstack([gy, gx]))
            ax = tps.interpolate(wx)
            ay = tps.interpolate(wy)
            result.deltaxs_tps = wx
            result.deltays_tps = wy
            result.tps = tps
            if last:
                xs_s = gx.copy().astype(np.float32)
                xs_s[sel] = xs
                ys_s = gy.copy().astype(np.float32)
                ys_s[sel] = ys
                dxs_full = ax.copy()
                dxs_full[sel] = sx
                dys_full = ay.copy()
                dys_full[sel] = sy
                result.xs_smooth = xs_s
                result.ys_smooth = ys_s
                result.deltaxs_smooth = dxs_full
                result.deltays_smooth = dys_full
    if not use_tps:
        ax = griddata(centers[::-1], dxs, ixvecs, iyvecs)
        ay = griddata(centers[::-1], dys, ixvecs, iyvecs)
    if last:
        result.deltaxs_final = ax
        result.deltays_final = ay
    else:
        result.deltaxs_approx = ax
        result.deltays_approx = ay
    return result


# ----------------------------------------------------------------------------------
# a16: multipass — works/piv/multipass.py:107-190
# ----------------------------------------------------------------------------------
def pass_shapes(shape_crop0, number, coeff_zoom=2):
    """Window shape of each pass: ``shape / coeff_zoom`` then ``int`` (multipass.py:153-165)."""
    if isinstance(shape_crop0, (int, np.integer)):
        shape = (shape_crop0, shape_crop0)
    else:
        shape = tuple(shape_crop0)
    coeffs = [coeff_zoom] * (number - 1) if isinstance(coeff_zoom, int) else list(coeff_zoom)
    shapes = [tuple(int(s) for s in shape)]
    for i in range(1, number):
        shape = (shape[0] / coeffs[i - 1], shape[1] / coeffs[i - 1])
        shapes.append(tuple(int(s) for s in shape))
    return shapes


def multipass(im0, im1, params, dtype_complex=np.complex64, keep_planes=False):
    """``WorkPIV.calcul`` with TPS between passes (``use_tps=True``).

    ``params`` has the upstream parameter tree attributes (``piv0``, ``fix``,
    ``multipass``).  Returns the list of pass results.
    """
    p0 = params.piv0
    mp = params.multipass
    fx = params.fix
    shapes = pass_shapes(p0.shape_crop_im0, mp.number, mp.coeff_zoom)
    grids = [make_grid(im0.shape, s, p0.grid.overlap) for s in shapes]
    results = []
    prev = None
    nb_peaks = int(getattr(p0, "nb_peaks_to_search", 1))
    extra = dict(method_subpix=getattr(p0, "method_subpix", "2d_gaussian2"),
                 nsubpix=getattr(p0, "nsubpix", None), nb_peaks_to_search=nb_peaks)
    keep = keep_planes or nb_peaks > 1
    for ip, shape in enumerate(shapes):
        subpix = ip == mp.number - 1
        if ip == 0:
            res = piv_pass(im0, im1, shape, p0.grid.overlap, grid=grids[ip],
                           apply_subpix=subpix, displacement_max=p0.displacement_max,
                           particle_radius=p0.particle_radius,
                           dtype_complex=dtype_complex, keep_planes=keep,
                           **extra)
        else:
            apply_interp(prev, grids[ip], mp)
            dxin = np.round(prev.deltaxs_approx).astype("int32")
            dyin = np.round(prev.deltays_approx).astype("int32")
            res = piv_pass(im0, im1, shape, p0.grid.overlap, grid=grids[ip],
                           dxin=dxin, dyin=dyin, apply_subpix=subpix,
                           displacement_max=p0.displacement_max,
                           particle_radius=p0.particle_radius,
                           dtype_complex=dtype_complex, keep_planes=keep, **extra)
        fix(res, fx.correl_min, fx.threshold_diff_neighbour, fx.displacement_max)
        results.append(res)
        prev = res
    try:
        apply_interp(prev, grids[-1], mp, last=True)
    except InterpError:
        pass
    return results
