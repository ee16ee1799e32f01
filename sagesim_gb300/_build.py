"""Builds libsagesim_gb300.so in-tree with nvcc for sm_103a.

The library holds the CUDA tick kernels, the C-ABI engine, the NVRTC runtime
for compiled step functions and the host-side graph utilities. Translation
units compile in parallel; an up-to-date library is not rebuilt.
"""
import concurrent.futures as _cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libsagesim_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-Wall", "-I" + BUILD, "-I" + CSRC,
         "-I" + INCLUDE]
SOURCES = ["sg_kernels.cu", "sg_count.cu", "sg_engine.cu", "sg_batch.cu", "sg_server.cpp", "sg_step_rt.cpp",
           "sg_graphs.cpp", "sg_noalloc.cu", "sg_setup.cu"]
HEADERS = ["sg_kernels.h", "sg_device.cuh", "sg_setup.h", "sg_internal.h", "sg_philox.h", "sg_step_rt.h", "sg_batch.h",
           "sg_count_flat.cuh"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build sagesim_gb300")


def _embed_headers():
    """Writes the NVRTC prelude (Philox + step API headers) as C++ raw strings."""
    out = os.path.join(BUILD, "sg_embedded_headers.h")
    parts = [("kSgPhiloxHeader", os.path.join(CSRC, "sg_philox.h")),
             ("kSgStepHeader", os.path.join(INCLUDE, "sagesim_gb300_step.h"))]
    text = ["// generated by sagesim_gb300/_build.py -- do not edit\n#pragma once\n"]
    for name, path in parts:
        body = open(path).read()
        if ")SGHDR\"" in body:
            raise RuntimeError("header contains the raw-string delimiter")
        text.append('static const char %s[] = R"SGHDR(%s)SGHDR";\n' % (name, body))
    new = "".join(text)
    if not os.path.exists(out) or open(out).read() != new:
        with open(out, "w") as f:
            f.write(new)
    return out


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    emb = _embed_headers()
    nvcc = _nvcc()
    common = [os.path.join(CSRC, h) for h in HEADERS] + [emb, os.path.join(INCLUDE, "sagesim_gb300.h"),
                                                          os.path.join(INCLUDE, "sagesim_gb300_step.h"),
                                                          __file__]
    jobs = []
    objs = []
    for src in _sources():
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + common):
            jobs.append([nvcc] + ARCH + FLAGS + ["-c", path, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stdout + r.stderr

    if jobs:
        with _cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or _stale(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-ldl", "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
