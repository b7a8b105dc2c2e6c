#!/usr/bin/env python3
"""Compile the reference's own device code, per pin case, into oracle/_ref/<case>.cubin.

TEST INFRASTRUCTURE ONLY.  Reads the reference sources where they lie (the directory given by
--reference, else $RBTP_REFERENCE_DIR, else /root/reference; present only on the development
machine), compiles them with nvcc for sm_103a (-rdc, the reference's
-std=c++14 raised to c++17 because CUDA 13's headers require it) against a generated parameters.h,
and device-links the objects into one cubin.  Nothing is copied from the reference: outputs go to
oracle/_ref/ only (git-ignored), and the cubin travels to GPU hosts as a build artefact.  The host
half of the reference (main.cu's loop, the particle wrappers) is restated by ref_driver.cpp.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import cases  # noqa: E402

DEFAULT_REF = "/root/reference"
REF = os.environ.get("RBTP_REFERENCE_DIR") or DEFAULT_REF


def reference_dir() -> str:
    """The reference source tree this recipe reads (see the module docstring)."""
    return REF
OUT = os.path.join(os.path.dirname(HERE), "_ref")
# main.cu and output/*.cu launch macrovar/collision/streaming and compute_Ked/ted; compiling them
# keeps those kernels referenced so the device link does not discard them.
SOURCES = ["main.cu", "output/output_flow.cu", "output/output_statis.cu", "output/output_part.cu",
           "src_lbm/globals.cu", "src_lbm/initial.cu", "src_lbm/collision.cu", "src_lbm/streaming.cu",
           "src_lbm/macrovar.cu", "src_part/pinit.cu", "src_part/links.cu", "src_part/refill.cu",
           "src_part/ibb.cu", "src_part/pforces.cu", "src_part/move.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def build_case(case: str) -> str:
    cdir = os.path.join(OUT, case)
    os.makedirs(os.path.join(cdir, "obj"), exist_ok=True)
    cubin = os.path.join(OUT, case + ".cubin")
    ph = os.path.join(cdir, "parameters.h")
    text = cases.parameters_h(case)
    if os.path.exists(cubin) and os.path.exists(ph) and open(ph).read() == text:
        newest = max(os.path.getmtime(p) for p in
                     [os.path.join(REF, s) for s in SOURCES] + [ph] +
                     [os.path.join(REF, "include", h) for h in os.listdir(os.path.join(REF, "include"))])
        if os.path.getmtime(cubin) >= newest:
            return cubin                      # up to date
    with open(ph, "w") as fh:
        fh.write(text)
    objs = []
    cmds = []
    for src in SOURCES:
        o = os.path.join(cdir, "obj", src.replace("/", "_").replace(".cu", ".o"))
        objs.append(o)
        cmds.append(["nvcc"] + ARCH + ["-O3", "-std=c++17", "-rdc=true", "-I" + cdir,
                                       "-I" + os.path.join(REF, "include"), "-I" + REF,
                                       "-c", os.path.join(REF, src), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for r in ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), cmds):
            if r.returncode != 0:
                raise RuntimeError("reference compile failed:\n" + r.stdout + r.stderr)
    r = subprocess.run(["nvcc"] + ARCH + ["-dlink", "-cubin", "-o", cubin] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("device link failed:\n" + r.stdout + r.stderr)
    for o in objs:  # host objects are not needed past the device link
        os.remove(o)
    return cubin


def main() -> int:
    global REF
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="reference source tree (default: $RBTP_REFERENCE_DIR "
                    "or " + DEFAULT_REF + ")")
    a = ap.parse_args()
    if a.reference:
        REF = a.reference
    if not os.path.isdir(REF):
        print("reference sources not present; nothing to build")
        return 0
    for case in list(cases.CASES) + list(cases.TIMING):
        print("built", build_case(case))
    return 0


if __name__ == "__main__":
    sys.exit(main())
