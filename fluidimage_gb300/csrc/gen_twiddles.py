"""Write ``fi_twiddles.cuh``: FFT twiddle factors as compile-time float constants.

``W_L^j = exp(-2 pi i j / L)`` for the base lengths L = 64 (covers 2, 4, ..., 64)
and L = 48 (covers 3, 6, 12, 24, 48), computed in double precision and rounded to
float32.  The header exposes ``constexpr`` switch functions so that, with the FFT
loops fully unrolled, every twiddle is an immediate operand.

Run: ``python fluidimage_gb300/csrc/gen_twiddles.py`` (the header is committed).
"""

import math
import struct
from pathlib import Path


def f32_literal(x: float) -> str:
    y = struct.unpack("f", struct.pack("f", x))[0]
    if y == 0.0:
        return "0.0f" if math.copysign(1.0, y) > 0 else "-0.0f"
    return f"{y.hex()}f".replace("0x", "0x")


def table(name: str, length: int) -> str:
    lines = [f"// W_{length}^j = exp(-2 pi i j / {length}); re = cos, im = -sin"]
    for part, fn in (("re", lambda j: math.cos(2 * math.pi * j / length)),
                     ("im", lambda j: -math.sin(2 * math.pi * j / length))):
        lines.append(f"__host__ __device__ constexpr float {name}_{part}(int j) {{")
        lines.append("  switch (j) {")
        for j in range(length):
            v = fn(j)
            # exact values at the quarter turns
            if j * 4 % length == 0:
                v = round(v)
            lines.append(f"    case {j}: return {f32_literal(v)};")
        lines.append("    default: return 0.0f;")
        lines.append("  }")
        lines.append("}")
    return "\n".join(lines)


def main():
    out = Path(__file__).with_name("fi_twiddles.cuh")
    text = "\n".join([
        "// Generated by gen_twiddles.py — do not edit.",
        "#pragma once",
        "",
        table("fi_tw64", 64),
        "",
        table("fi_tw48", 48),
        "",
    ])
    out.write_text(text)
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
