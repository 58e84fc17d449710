"""Builds the oracle's reference libraries from the reference's own sources.

Test infrastructure only.  Compiles the reference's preprocessing and
reconstruction source files where they lie (REF, default /root/reference)
with g++, against the stand-in headers in shim/ (FFTW3 implemented by
fftw_shim.cpp; OpenCV and libtiff declared only), together with the drivers
ref_pretraitement.cpp and ref_reconstruction.cpp, into
oracle/_ref/libref_pretraitement.so and oracle/_ref/libref_reconstruction.so.
Functions of those source files that the drivers never reach may call into
OpenCV, libtiff or other translation units that are not built; each such
symbol is given a definition that aborts, so that the libraries load.

    python oracle/ref/build_ref.py [REF]
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
FLAGS = ["-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-w"]

LIBS = {
    "libref_pretraitement.so": {
        "dir": "Tomo_prog/pretraitement_hors_axe_CPU",
        "includes": [".", "include"],
        "sources": ["fonctions.cpp", "FFT_fonctions.cpp", "src/deroulement_volkov4.cpp", "src/FFTW_init.cpp",
                    "src/vecteur.cpp", "deroulement_herraez.cpp"],
        "driver": "ref_pretraitement.cpp",
    },
    "libref_reconstruction.so": {
        "dir": "Tomo_prog/Reconstruction",
        "includes": ["include"],
        "sources": ["src/fonctions.cpp", "src/FFT_fonctions.cpp", "src/FFT_encaps.cpp", "src/manip.cpp",
                    "src/Point2D.cpp", "src/Point3D.cpp"],
        "driver": "ref_reconstruction.cpp",
    },
}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode, r.stdout + r.stderr


def _build(name, spec, ref):
    base = os.path.join(ref, spec["dir"])
    obj_dir = os.path.join(OUT, "obj", name)
    os.makedirs(obj_dir, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "shim")] + sum((["-I", os.path.join(base, d)] for d in spec["includes"]), [])
    srcs = [os.path.join(base, s) for s in spec["sources"]]
    srcs += [os.path.join(HERE, spec["driver"]), os.path.join(HERE, "fftw_shim.cpp")]
    objs = []
    for s in srcs:
        o = os.path.join(obj_dir, os.path.basename(os.path.dirname(s)) + "_" + os.path.basename(s) + ".o")
        rc, log = _run(["g++"] + FLAGS + inc + ["-c", s, "-o", o])
        if rc:
            raise RuntimeError(f"compiling {s} failed:\n{log}")
        objs.append(o)
    lib = os.path.join(OUT, name)
    link = ["g++", "-shared", "-fopenmp", "-o", lib] + objs
    # symbols the built files reference but do not define: definitions that abort
    rc, log = _run(link + ["-Wl,--no-undefined", "-Wl,--no-demangle"])
    missing = sorted(set(re.findall(r"undefined reference to `([^']+)'", log)))
    if rc and not missing:
        raise RuntimeError(f"linking {name} failed:\n{log}")
    if missing:
        stub = os.path.join(obj_dir, "unbuilt_symbols.c")
        with open(stub, "w") as f:
            f.write("/* Functions of translation units that are not built; never reached by the drivers. */\n")
            f.write("#include <stdlib.h>\n")
            for m in missing:
                f.write(f"void {m}(void) {{ abort(); }}\n")
        so = stub[:-2] + ".o"
        rc, log = _run(["gcc", "-fPIC", "-c", stub, "-o", so])
        if rc:
            raise RuntimeError(log)
        rc, log = _run(link + [so, "-Wl,--no-undefined"])
        if rc:
            raise RuntimeError(f"linking {name} failed:\n{log}")
    return lib


def build(ref: str | None = None) -> list[str]:
    ref = ref or os.environ.get("TDM_REFERENCE", "/root/reference")
    if not os.path.isdir(os.path.join(ref, "Tomo_prog")):
        return []
    os.makedirs(OUT, exist_ok=True)
    return [_build(n, s, ref) for n, s in LIBS.items()]


if __name__ == "__main__":
    for p in build(sys.argv[1] if len(sys.argv) > 1 else None):
        print(p)
