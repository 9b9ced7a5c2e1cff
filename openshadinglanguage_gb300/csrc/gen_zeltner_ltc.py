"""Writes oslg_zeltner_ltc.inc: the 32 x 32 table of linearly transformed
cosine coefficients (A, B, R) per (roughness, cos theta_o) of the
Zeltner-Burley-Chiang sheen model ("Practical Multiple-Scattering Sheen
Using Linearly Transformed Cosines", SIGGRAPH 2022), as the reference's
BSDL carries it (libbsdl MTX/bsdf_zeltnersheen_param.h). The table is
published fit data that sheen_bsdf's "mode" 1 interpolates; results must
use the same numbers, so they are read from the reference tree here.

Usage: python gen_zeltner_ltc.py [REFERENCE_SOURCE_TREE]
(default $OSL_REFERENCE_ROOT, else /root/reference).
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OSL_REFERENCE_ROOT", "/root/reference")
    src = open(os.path.join(ref, "src/libbsdl/include/BSDL/MTX/bsdf_zeltnersheen_param.h")).read()
    body = src.split("// clang-format off")[1].split("// clang-format on")[0]
    triples = re.findall(r"\{\s*(-?[0-9.eE+-]+)\s*,\s*(-?[0-9.eE+-]+)\s*,\s*(-?[0-9.eE+-]+)\s*\}", body)
    assert len(triples) == 32 * 32, len(triples)
    lines = ["// generated by gen_zeltner_ltc.py: Zeltner et al. 2022 sheen LTC coefficients (A, B, R),",
             "// 32 rows of roughness x 32 columns of cos(theta_o), row-major"]
    for r in range(32):
        row = triples[r * 32:(r + 1) * 32]
        lines.append(", ".join("%sf, %sf, %sf" % t for t in row) + ",")
    open(os.path.join(HERE, "oslg_zeltner_ltc.inc"), "w").write("\n".join(lines) + "\n")
    print("wrote", len(triples), "entries")


if __name__ == "__main__":
    main()
