"""The algebra of the tensor-core correlation pass, checked on the CPU.

``tc_emulation`` follows fi_correl_tc.cu stage by stage (packed real DFT of the
rows, column DFT of [Re | Im] with kx = 0 and 16 sharing one complex row, the
Hermitian separation before the cross spectrum, the inverse, the Hermitian-weighted
real inverse, the power-of-two scales).  Without operand splitting it must equal
numpy's FFT correlation (``ifft2(conj(F0) F1).real``, ``F[0,0] = 0``) to float32
rounding of the intermediate operands; with the forms' splits, the plane error
relative to the plane maximum must stay within each form's bound: bf16 x1 1e-2,
bf16 3-term 2e-5, fp16 3-term 1e-6 (predicted ~2e-3, ~3e-6, ~1.2e-7).
"""

import numpy as np
import pytest

import tc_emulation as T

BOUNDS = {None: 1e-7, "bf16x1": 1e-2, "bf16x3": 2e-5, "fp16x3": 1e-6}


def _windows(dtype, seed):
    from fluidimage_gb300 import synthetic

    if dtype == "uint16":
        model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0), intensity=(1000, 4000),
                                        noise=20.0, dtype="uint16", max_value=4095)
    else:
        model = synthetic.ParticleModel(density=0.05, noise=2.0, dtype="uint8")
    im0, im1 = synthetic.make_pair((160, 160), synthetic.uniform_shift(3.3, -5.7), model,
                                   seed=seed)
    out = []
    for y, x in ((8, 8), (60, 90), (110, 30)):
        out.append((im0[y:y + 32, x:x + 32].astype(np.float64),
                    im1[y:y + 32, x:x + 32].astype(np.float64)))
    return out


@pytest.mark.parametrize("form", [None, "bf16x1", "bf16x3", "fp16x3"])
@pytest.mark.parametrize("dtype", ["uint8", "uint16"])
def test_emulated_planes_match_fft(form, dtype):
    for w0, w1 in _windows(dtype, 11):
        ref = T.reference_plane(w0, w1)
        got = T.correl_plane(w0, w1, form)
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err <= BOUNDS[form], (form, err)
        assert np.argmax(got) == np.argmax(ref)


def test_emulation_flat_and_bright_windows():
    """A constant window gives a zero plane; a 16-bit window near 65535 keeps the FP16
    operands finite (input scaled below 2^15) and stays as accurate as a float32 FFT
    of the same windows (the mean dominates: float32 rounding of the DC column)."""
    rng = np.random.default_rng(3)
    w1 = rng.integers(0, 4096, (32, 32)).astype(np.float64)
    flat = np.full((32, 32), 17.0)
    assert np.abs(T.correl_plane(flat, w1, "fp16x3")).max() < 1e-9 * np.abs(w1).max() ** 2
    bright0 = 65535.0 - rng.integers(0, 40, (32, 32))
    bright1 = np.roll(bright0, 2, axis=1)
    ref = T.reference_plane(bright0, bright1)
    got = T.correl_plane(bright0, bright1, "fp16x3")
    assert np.isfinite(got).all()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    err32 = np.abs(T.reference_plane(bright0, bright1, np.complex64) - ref).max() / np.abs(ref).max()
    assert err < max(err32, 1e-4), (err, err32)
