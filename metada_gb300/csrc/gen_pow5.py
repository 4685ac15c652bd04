"""Writes mg_pow5.h: for every decimal exponent q in [-342, 308], the 128
most significant bits of 5^q (q >= 0: truncated), or of 2^(b + 127) / 5^-q
with b the bit length of 5^-q (q < 0: rounded up), as two 64-bit words.
This is the table of the Eisel-Lemire decimal-to-binary conversion
(D. Lemire, "Number Parsing at a Gigabyte per Second", Software: Practice
and Experience 51(8), 2021), computed here with exact integers.

    python metada_gb300/csrc/gen_pow5.py   (rewrites mg_pow5.h beside it)
"""
from pathlib import Path

QMIN, QMAX = -342, 308


def entry(q: int) -> int:
    if q >= 0:
        v = 5 ** q
        b = v.bit_length()
        return v >> (b - 128) if b > 128 else v << (128 - b)
    v = 5 ** (-q)
    b = v.bit_length()
    return (1 << (b + 127)) // v + 1


def render() -> str:
    lines = [
        "// Generated by gen_pow5.py: do not edit.  128-bit significands of 5^q",
        f"// for q in [{QMIN}, {QMAX}] (high word, low word), the table of the",
        "// Eisel-Lemire conversion in mg_io.cu.",
        "#pragma once",
        "#include <stdint.h>",
        "",
        f"#define MG_POW5_QMIN ({QMIN})",
        f"#define MG_POW5_QMAX ({QMAX})",
        "",
        f"__device__ const uint64_t kPow5Table[{2 * (QMAX - QMIN + 1)}] = {{",
    ]
    for q in range(QMIN, QMAX + 1):
        t = entry(q)
        assert (1 << 127) <= t < (1 << 128)
        lines.append(f"    0x{t >> 64:016x}ull, 0x{t & ((1 << 64) - 1):016x}ull,  // {q}")
    lines.append("};")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    (Path(__file__).resolve().parent / "mg_pow5.h").write_text(render())
