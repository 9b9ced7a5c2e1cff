"""ORACLE build recipe (test infrastructure only).

Compiles the CPU restatement in this folder into oracle/_build/liboslg_oracle.so
with floating-point contraction disabled (-ffp-contract=off), so its float
operations are the non-FMA reference order on every host (x86 and AArch64
alike). OpenMP parallelises the per-point loop for the CPU baseline.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboslg_oracle.so")
SOURCES = ["oracle.cpp", "oracle_wavefront.cpp"]
HEADERS = sorted(f for f in os.listdir(HERE) if f.endswith(".h"))


def _product_build():
    """The product's build recipe, loaded by path (not through the package)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "_oslg_product_build", os.path.join(HERE, "..", "openshadinglanguage_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [os.path.join(HERE, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(HERE, "..", "openshadinglanguage_gb300", "csrc", "oslg_program.h"))
    deps.append(os.path.join(HERE, "..", "include", "oslg.h"))
    deps.append(os.path.join(HERE, "..", "openshadinglanguage_gb300", "csrc", "oslg_zeltner_ltc.inc"))
    # the BSDL energy tables the product bakes (data shared with the oracle)
    deps.append(_product_build().bsdl_luts())
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-Wall", "-Wno-unused-function", "-o", LIB] + [os.path.join(HERE, s) for s in SOURCES]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
