"""Builds the engine's shared library for sm_103a with nvcc (no torch needed).

The library is built in-tree (pi-qmc_gb300/pimc_gb300/libpimc_gb300.so, git-ignored)
so that it is found by path and never silently replaced by another copy.
"""
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
LIB = os.path.join(PKG, "libpimc_gb300.so")
# (source, extra flags): the section kernel's register-budget variants are
# separate objects so that nvcc compiles them in parallel
SOURCES = [("engine.cu", []), ("tables.cc", []), ("paths_io.cc", [])] + [
    ("section_variants.cu", [f"-DPIMC_NT={nt}", f"-DPIMC_MINB={v}"])
    for nt, v in ((256, 2), (256, 3), (256, 4), (512, 1))] + [
    # the variants without the fixed-node phases (launches without node models)
    ("section_variants.cu", ["-DPIMC_NT=256", f"-DPIMC_MINB={v}", "-DPIMC_NODES=0"])
    for v in (2, 3, 4)]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    hdr = os.path.join(os.path.dirname(ROOT), "include", "pimc_gb300.h")
    return os.path.exists(hdr) and os.path.getmtime(hdr) > t


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    objs = []
    procs = []
    for src, flags in SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        tag = "".join(f.split("=")[-1] for f in flags)
        obj = os.path.join(PKG, "_build_" + src.replace(".", "_") + tag + ".o")
        if src.endswith(".cu"):
            cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", *flags, "-c", path, "-o", obj]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", path,
                   "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT, text=True)))
        objs.append(obj)
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + out)
        if verbose and out.strip():
            print(out)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stderr)
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
