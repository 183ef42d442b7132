"""Build recipe for the native libraries of pargo_gb300 (in-tree, no cmake).

* ``lib/libpargo_gpu.so``   -- the CUDA kernels + the C ABI of include/pargo_gpu.h,
  compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``).
* ``lib/libpargo_synth.so`` -- the seeded synthetic-DEM generator (host C).
* ``lib/libpargo_gpro.so`` and ``lib/bin/*`` -- the gpro-compatible C++ host
  layer and the slope / D8 / pit-remove / SCA application mains built on it.

Translation units compile in parallel; a full build takes well under a minute.
Host code uses ``-ffp-contract=off`` so x86-64 and aarch64 builds compute
identical bytes.
"""
import os
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
GPRO = os.path.join(PKG, "gpro")
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(LIB, "obj")
BIN = os.path.join(LIB, "bin")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-I" + INCLUDE]
CU_SOURCES = ["abi.cu", "focal.cu", "focal64.cu", "fill.cu", "sca.cu", "sca_tiled.cu", "twi.cu", "mfd.cu", "load.cu", "grad.cu", "noalloc.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _run_all(cmds):
    procs = [(name, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for name, c in cmds]
    errors = []
    for name, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append("%s failed:\n%s\n%s" % (name, " ".join(cmds[[n for n, _ in cmds].index(name)][1]),
                                                   out.decode(errors="replace")))
    if errors:
        raise RuntimeError("\n".join(errors))


def gpro_sources():
    src = os.path.join(GPRO, "src")
    if not os.path.isdir(src):
        return []
    return sorted(os.path.join(src, f) for f in os.listdir(src) if f.endswith(".cpp"))


def app_sources():
    apps = os.path.join(GPRO, "apps")
    if not os.path.isdir(apps):
        return []
    return sorted(os.path.join(apps, f) for f in os.listdir(apps) if f.endswith(".cpp"))


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    cmds = []
    objs = []
    for src in CU_SOURCES:
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        cmds.append((src, [nvcc()] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", o]))
    cmds.append(("synth", ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                           os.path.join(CSRC, "synth.c"), "-o", os.path.join(LIB, "libpargo_synth.so")]))
    gsrc = gpro_sources()
    gobjs = []
    for src in gsrc:
        o = os.path.join(OBJ, "gpro_" + os.path.basename(src).replace(".cpp", ".o"))
        gobjs.append(o)
        cmds.append((os.path.basename(src), ["g++", "-std=c++14", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                                             "-I" + INCLUDE, "-I" + os.path.join(GPRO, "include"), "-c", src, "-o", o]))
    _run_all(cmds)
    link = [(
        "libpargo_gpu.so",
        [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC"] + objs + ["-o", os.path.join(LIB, "libpargo_gpu.so")],
    )]
    _run_all(link)
    if gobjs:
        gpro_so = os.path.join(LIB, "libpargo_gpro.so")
        _run_all([("libpargo_gpro.so", ["g++", "-shared", "-o", gpro_so] + gobjs +
                   ["-L" + LIB, "-lpargo_gpu", "-Wl,-rpath,$ORIGIN"])])
        apps = []
        for src in app_sources():
            exe = os.path.join(BIN, os.path.basename(src).replace(".cpp", ""))
            apps.append((os.path.basename(src), ["g++", "-std=c++14", "-O2", "-ffp-contract=off", "-Wall",
                                                 "-I" + INCLUDE, "-I" + os.path.join(GPRO, "include"), src, "-o", exe,
                                                 "-L" + LIB, "-lpargo_gpro", "-lpargo_gpu",
                                                 "-Wl,-rpath,$ORIGIN/.."]))
        if apps:
            _run_all(apps)
    if verbose:
        print("built", LIB)


if __name__ == "__main__":
    build(verbose=True)
