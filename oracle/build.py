"""Build recipe for the test oracle (test infrastructure only).

Two libraries:

* ``oracle/_build/liboracle.so`` -- the C restatement ``oracle/pargo_oracle.c``.
  Built on every machine (it is what the GPU parity tests and the CPU
  baseline use).
* ``oracle/_ref/libpargo_ref.so`` -- the UNMODIFIED reference operators,
  compiled from the reference sources where they lie (``gpro/application.cpp``,
  ``gpro/utility.cpp``, the ``apps/.../*Operator.cpp`` of the path) against the
  single-rank ``mpi.h`` and in-memory ``gdal_priv.h`` in ``oracle/ref_shim/``,
  plus ``oracle/ref_driver.cpp``.  Built only where the reference tree exists.
  Nothing is copied out of the reference; only the objects land in
  ``oracle/_ref/``.

Both use ``-ffp-contract=off``: the reference is plain IEEE double arithmetic
and must not pick up fused multiply-adds (GCC contracts by default on aarch64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD, "liboracle.so")
REF_SO = os.path.join(REF_OUT, "libpargo_ref.so")
REF_MFD_SO = os.path.join(REF_OUT, "libpargo_ref_mfd.so")
REFERENCE_ROOT = os.environ.get("PARGO_REFERENCE_ROOT", "/root/reference")

REF_SOURCES = [
    "gpro/application.cpp",
    "gpro/utility.cpp",
    "apps/morphology/slope/slopeOperator.cpp",
    "apps/hydrology/flowdird8/d8Operator.cpp",
    "apps/hydrology/pitremove/pitRemoveOperator.cpp",
    "apps/hydrology/scad8/scaOperator.cpp",
    "apps/hydrology/twi/TWIOperator.cpp",
]
REF_INCLUDES = [
    "gpro",
    "apps/morphology/slope",
    "apps/hydrology/flowdird8",
    "apps/hydrology/pitremove",
    "apps/hydrology/scad8",
    "apps/hydrology/twi",
]


def oracle_cmd():
    os.makedirs(BUILD, exist_ok=True)
    return ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
            os.path.join(HERE, "pargo_oracle.c"), "-o", ORACLE_SO, "-lm"]


# The MFD-md pair lives in a library of its own: its SCA operator has the
# same class name as the D8 one.
REF_MFD_SOURCES = [
    "gpro/application.cpp",
    "gpro/utility.cpp",
    "apps/hydrology/flowdirmfdmd/mfdOperator.cpp",
    "apps/hydrology/scamfdmd/scaOperator.cpp",
]
REF_MFD_INCLUDES = ["gpro", "apps/hydrology/flowdirmfdmd", "apps/hydrology/scamfdmd"]


def reference_available():
    return all(os.path.exists(os.path.join(REFERENCE_ROOT, s)) for s in REF_SOURCES)


def ref_cmd():
    os.makedirs(REF_OUT, exist_ok=True)
    cmd = ["g++", "-std=gnu++14", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-DLINUX", "-DNDEBUG", "-w", "-I" + os.path.join(HERE, "ref_shim")]
    cmd += ["-I" + os.path.join(REFERENCE_ROOT, d) for d in REF_INCLUDES]
    cmd += [os.path.join(REFERENCE_ROOT, s) for s in REF_SOURCES]
    cmd += [os.path.join(HERE, "ref_driver.cpp"), "-o", REF_SO]
    return cmd


def ref_mfd_cmd():
    os.makedirs(REF_OUT, exist_ok=True)
    cmd = ["g++", "-std=gnu++14", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-DLINUX", "-DNDEBUG", "-w", "-I" + os.path.join(HERE, "ref_shim")]
    cmd += ["-I" + os.path.join(REFERENCE_ROOT, d) for d in REF_MFD_INCLUDES]
    cmd += [os.path.join(REFERENCE_ROOT, s) for s in REF_MFD_SOURCES]
    cmd += [os.path.join(HERE, "ref_driver_mfd.cpp"), "-o", REF_MFD_SO]
    return cmd


def commands():
    """(name, argv) pairs for everything buildable on this machine."""
    out = [("oracle", oracle_cmd())]
    if reference_available():
        out.append(("reference", ref_cmd()))
        if all(os.path.exists(os.path.join(REFERENCE_ROOT, s)) for s in REF_MFD_SOURCES):
            out.append(("reference MFD-md", ref_mfd_cmd()))
    return out


def build(verbose=False):
    procs = [(n, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for n, c in commands()]
    for n, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build step %r failed:\n%s" % (n, out.decode(errors="replace")))
        if verbose and out:
            sys.stdout.write(out.decode(errors="replace"))


if __name__ == "__main__":
    build(verbose=True)
    print("built", ORACLE_SO, REF_SO if reference_available() else "(reference tree absent)")
