"""Build the reference's own kernels as a host shared library (oracle/_ref/).

TEST INFRASTRUCTURE ONLY.  Reads the reference sources where they lie
(rupertnash/gpu-swimmers: lbswim/liblbswim/{Shared,lb,SwimmerArray,
TracerArray}.cu, in the order of lbswim.cu), rewrites each ``K<<<g, b>>>(args);``
launch into ``ref_launch(g, b, [&]{ K(args); });``, appends
oracle/ref_shim/ref_driver.inc and pipes the result straight into g++.  No
copy of a reference source is written to disk; the only output is
oracle/_ref/libref.so.  The cuRAND header is replaced by
oracle/ref_shim/curand_kernel.h (the project's counter-based stream), and the
shim header makes __global__/__device__ empty.

Usage: python oracle/build_ref.py [REFERENCE_ROOT]   (default: $LBSWIM_REFERENCE_ROOT)
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# Where the reference checkout lies: $LBSWIM_REFERENCE_ROOT, else the path of
# this build machine's read-only copy.
DEFAULT_REF = os.environ.get("LBSWIM_REFERENCE_ROOT", "/root/reference")
SOURCES = ["Shared.cu", "lb.cu", "SwimmerArray.cu", "TracerArray.cu"]
LAUNCH = re.compile(r"(\w+)\s*<<<(.*?)>>>\s*\((.*?)\)\s*;", re.S)


def translate(text):
    return LAUNCH.sub(lambda m: "ref_launch(%s, [&]{ %s(%s); });" % (m.group(2), m.group(1), m.group(3)), text)


def reference_root():
    """The reference checkout if its kernel sources are present, else None
    (machines without the reference skip everything that needs it)."""
    return DEFAULT_REF if os.path.isdir(os.path.join(DEFAULT_REF, "lbswim", "liblbswim")) else None


def build(ref_root=DEFAULT_REF, out_dir=None, quiet=False):
    lib_dir = os.path.join(ref_root, "lbswim", "liblbswim")
    if not os.path.isdir(lib_dir):
        raise FileNotFoundError("reference sources not found at %s" % lib_dir)
    out_dir = out_dir or os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    parts = []
    for name in SOURCES:
        with open(os.path.join(lib_dir, name)) as fh:
            parts.append('#line 1 "%s"\n' % name + translate(fh.read()))
    with open(os.path.join(HERE, "ref_shim", "ref_driver.inc")) as fh:
        parts.append('#line 1 "ref_driver.inc"\n' + fh.read())
    unit = "\n".join(parts)
    out = os.path.join(out_dir, "libref.so")
    # The counter-based RNG the cuRAND stand-in calls lives in the oracle's C file.
    obj = os.path.join(out_dir, "rng_oracle.o")
    subprocess.run(["gcc", "-c", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c11",
                    os.path.join(HERE, "lbswim_oracle.c"), "-o", obj], check=True)
    cmd = ["g++", "-x", "c++", "-", "-x", "none", obj, "-O2", "-fPIC", "-shared", "-fopenmp",
           "-std=c++17", "-ffp-contract=off", "-ftrivial-auto-var-init=zero", "-w",
           "-include", os.path.join(HERE, "ref_shim", "cuda_host_shim.h"),
           "-I", os.path.join(HERE, "ref_shim"), "-I", lib_dir, "-o", out]
    subprocess.run(cmd, input=unit.encode(), check=True)
    if not quiet:
        print("built", out)
    return out


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF)
