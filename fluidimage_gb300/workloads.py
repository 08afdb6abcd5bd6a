"""Synthetic PIV workloads used by the tests and the benchmark.

``config1``: one 512x512 pair, float32 built from uint8, uniform shift (3.3, -1.7),
32 px windows, overlap 0.5, '2d_gaussian2', no neighbour filter.
``config2``: one 2048x2048 uint16 (12-bit) pair, Oseen vortex (rc = 200 px, peak
8 px), noise 20 counts; three passes 64 -> 32 -> 16 px, overlap 0.5, neighbour
threshold 2, TPS between passes (subdomains of 200 vectors, smoothing 0.5).
Seeds follow ``seed = config_index * 1000 + pair_index``.
"""

from __future__ import annotations

from . import synthetic


def config1_images(pair=0, shape=(512, 512)):
    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0), intensity=(128, 255),
                                    noise=2.0, dtype="uint8")
    field = synthetic.uniform_shift(3.3, -1.7)
    return synthetic.make_pair(shape, field, model, seed=1000 + pair, as_float32=True), field


def config1_params(params):
    params.piv0.shape_crop_im0 = 32
    params.piv0.grid.overlap = 0.5
    params.piv0.method_subpix = "2d_gaussian2"
    params.multipass.number = 1
    params.fix.threshold_diff_neighbour = None
    params.fix.correl_min = float("-inf")
    return params


def config2_images(pair=0, shape=(2048, 2048)):
    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0), intensity=(1000, 4000),
                                    noise=20.0, dtype="uint16", max_value=4095)
    field = synthetic.oseen_vortex(shape, d_max=8.0, rc=200.0)
    return synthetic.make_pair(shape, field, model, seed=2000 + pair), field


def config2_params(params):
    params.piv0.shape_crop_im0 = 64
    params.piv0.grid.overlap = 0.5
    params.multipass.number = 3
    params.multipass.coeff_zoom = 2
    params.multipass.use_tps = True
    params.multipass.subdom_size = 200
    params.multipass.smoothing_coef = 0.5
    params.fix.threshold_diff_neighbour = 2
    return params


def config4_images(pair=0, shape=(4096, 4096)):
    """Precision-sweep pair: uint16 12-bit, density 0.06 particles/px, diameter 2.5 px,
    noise 1 % of the maximum, d = 5 (sin(2 pi y / 512), cos(2 pi x / 512)) px."""
    model = synthetic.ParticleModel(density=0.06, diameter=(2.5, 2.5), intensity=(1000, 4000),
                                    noise=0.01 * 4095, dtype="uint16", max_value=4095)
    field = synthetic.sinusoid(5.0, 512.0)
    return synthetic.make_pair(shape, field, model, seed=4000 + pair), field


def config4_params(params):
    """One pass of 32 px windows at overlap 0.75 (509 x 509 = 259 081 vectors at
    4096^2), WorkFIX with neighbour threshold 2, final TPS on subdomains of 256
    vectors."""
    params.piv0.shape_crop_im0 = 32
    params.piv0.grid.overlap = 0.75
    params.multipass.number = 1
    params.multipass.use_tps = "last"
    params.multipass.subdom_size = 256
    params.multipass.smoothing_coef = 0.5
    params.fix.threshold_diff_neighbour = 2
    return params


CONFIG3_SIZES = ((512, 512), (768, 1024), (2048, 2048), (2160, 4096))
CONFIG3_WINDOWS = (16, 24, 32, 48, 64)
CONFIG3_OVERLAPS = (0.5, 0.75)


def _oseen_superposition(shape, rng, count=4, peak=6.0):
    """Sum of ``count`` Oseen vortices at random centres, core radii and signs, each
    of peak ``peak / count`` px (the sum stays below ``peak`` px)."""
    ny, nx = shape
    fields = []
    for _ in range(count):
        centre = (rng.uniform(0, nx), rng.uniform(0, ny))
        rc = rng.uniform(0.05, 0.2) * min(nx, ny)
        sign = rng.choice((-1.0, 1.0))
        fields.append((sign, synthetic.oseen_vortex(shape, d_max=peak / count, rc=rc,
                                                    center=centre)))

    def field_(x, y):
        dx = 0.0
        dy = 0.0
        for sign, f in fields:
            a, b = f(x, y)
            dx = dx + sign * a
            dy = dy + sign * b
        return dx, dy

    field_.max_displacement = peak
    return field_


def config3_pair(size_index, k, seed):
    """One image pair of the batched heterogeneous workload: uint16 12-bit, density
    U[0.02, 0.08], diameter U[2, 4] px; a uniform shift U[-6, 6]^2 px (even k) or a
    superposition of 4 Oseen vortices of peak <= 6 px (odd k)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    shape = CONFIG3_SIZES[size_index]
    model = synthetic.ParticleModel(density=rng.uniform(0.02, 0.08), diameter=(2.0, 4.0),
                                    intensity=(1000, 4000), noise=20.0, dtype="uint16",
                                    max_value=4095)
    if k % 2 == 0:
        field = synthetic.uniform_shift(*rng.uniform(-6.0, 6.0, 2))
    else:
        field = _oseen_superposition(shape, rng)
    return synthetic.make_pair(shape, field, model, seed=seed + 1)


def config3_jobs(params_factory, npairs=256, per_size=4, seed=3000):
    """The batched heterogeneous workload: ``npairs`` single-pass jobs (image size,
    window size and overlap drawn uniformly) over ``per_size`` distinct image pairs of
    each size; returns [(im0, im1, params)] (host arrays; the jobs of one image pair
    share its arrays) and the draws (shape, window, overlap)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    pool = {(s, k): config3_pair(s, k, seed + 100 * s + k)
            for s in range(len(CONFIG3_SIZES)) for k in range(per_size)}
    jobs, draws = [], []
    for _ in range(npairs):
        s = int(rng.integers(len(CONFIG3_SIZES)))
        k = int(rng.integers(per_size))
        n = int(rng.choice(CONFIG3_WINDOWS))
        ov = float(rng.choice(CONFIG3_OVERLAPS))
        params = params_factory()
        params.piv0.shape_crop_im0 = n
        params.piv0.grid.overlap = ov
        params.multipass.number = 1
        im0, im1 = pool[(s, k)]
        jobs.append((im0, im1, params))
        draws.append((CONFIG3_SIZES[s], n, ov))
    return jobs, draws


def config5_field(shape=(2048, 2048), peak=7.0):
    """Oseen vortex (rc 200 px) plus the sinusoid (sin 2 pi y / 512, cos 2 pi x / 512),
    scaled together so that the largest displacement is ``peak`` px."""
    import numpy as np

    oseen = synthetic.oseen_vortex(shape, d_max=1.0, rc=200.0)
    sinus = synthetic.sinusoid(1.0, 512.0)
    ys, xs = np.mgrid[0:shape[0]:4, 0:shape[1]:4].astype(np.float64)
    ou, ov = oseen(xs, ys)
    su, sv = sinus(xs, ys)
    scale = peak / float(np.hypot(ou + su, ov + sv).max())

    def field_(x, y):
        a, b = oseen(x, y)
        c, d = sinus(x, y)
        return scale * (a + c), scale * (b + d)

    field_.max_displacement = peak
    return field_


def config5_images(pair=0, shape=(2048, 2048)):
    """Refinement pair: the particle model of the multipass workload (uint16 12-bit,
    density 0.05, diameter U[2, 3] px, noise 20), the Oseen-plus-sinusoid field of
    peak 7 px; returned as float32 images and the field."""
    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0), intensity=(1000, 4000),
                                    noise=20.0, dtype="uint16", max_value=4095)
    field = config5_field(shape)
    im0, im1 = synthetic.make_pair(shape, field, model, seed=5000 + pair)
    return (im0.astype("float32"), im1.astype("float32")), field
