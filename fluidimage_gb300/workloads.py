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
