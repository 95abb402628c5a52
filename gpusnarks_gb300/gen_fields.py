"""Write csrc/fields_gen.h: per-field constants for host and device code.

Run ``python -m gpusnarks_gb300.gen_fields`` after changing fields.py.  The
generated header is committed; build() does not regenerate it.

Each field becomes a struct with ``constexpr`` accessor functions (device code
cannot index a ``static constexpr`` member array) holding the modulus, the
CIOS constant ``-p^-1 mod 2^32``, ``R mod p`` (Montgomery one) and
``R^2 mod p`` (to enter Montgomery form) for ``R = 2^(32*LIMBS)``.
"""
from __future__ import annotations

import pathlib

from .fields import FIELDS

OUT = pathlib.Path(__file__).resolve().parent / "csrc" / "fields_gen.h"


def _accessor(name: str, value: int, limbs: int) -> str:
    cases = []
    for i in range(limbs):
        cases.append(f"      case {i}: return 0x{(value >> (32 * i)) & 0xFFFFFFFF:08X}u;")
    body = "\n".join(cases)
    return (f"  __host__ __device__ static constexpr uint32_t {name}(int i) {{\n"
            f"    switch (i) {{\n{body}\n      default: return 0u;\n    }}\n  }}\n")


def render() -> str:
    parts = [
        "// Generated by gpusnarks_gb300/gen_fields.py from gpusnarks_gb300/fields.py.",
        "// Do not edit by hand.",
        "#pragma once",
        "#include <cstdint>",
        "",
        "#include \"gsn_compat.h\"",
        "",
        "namespace gsn {",
        "",
    ]
    struct_names = {"p32": "FieldP32", "bls12_381_fr": "FieldBLS12_381",
                    "mnt4753_fr": "FieldMNT4_753", "mnt4753_fq": "FieldMNT4_753_Q"}
    for f in FIELDS.values():
        R = f.R
        headroom = R // f.p  # how many copies of p fit below R
        parts.append(f"// {f.name}: {f.p.bit_length()}-bit modulus, {f.limbs} limb(s), "
                     f"2-adicity {f.two_adicity}, generator {f.generator}")
        parts.append(f"struct {struct_names[f.name]} {{")
        parts.append(f"  static constexpr int ID = {f.fid};")
        parts.append(f"  static constexpr int N = {f.limbs};")
        parts.append(f"  static constexpr uint32_t PINV = 0x{f.pinv:08X}u;")
        parts.append(f"  static constexpr int TWO_ADICITY = {f.two_adicity};")
        parts.append(f"  static constexpr uint32_t GENERATOR = {f.generator}u;")
        parts.append(f"  static constexpr int BITS = {f.p.bit_length()};")
        parts.append(f"  // floor(R / p): 1 means no headroom, >= 4 allows sums of two [0,2p) values.")
        parts.append(f"  static constexpr uint32_t HEADROOM = {min(headroom, 0xFFFFFFFF)}u;")
        parts.append(_accessor("mod", f.p, f.limbs))
        parts.append(_accessor("r1", R % f.p, f.limbs))
        parts.append(_accessor("r2", (R * R) % f.p, f.limbs))
        parts.append("};")
        parts.append("")
    parts.append("}  // namespace gsn")
    parts.append("")
    return "\n".join(parts)


def main() -> None:
    OUT.write_text(render())
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
