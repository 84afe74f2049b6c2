"""Builds the renderer's shared library in-tree: lighttransportsimulation_gb300/_lib/liblts_gb300.so.

CUDA sources are compiled for sm_103a only (`-gencode arch=compute_103a,code=sm_103a`) with
`-fmad=false`: no multiply-add is fused unless the source asks for it (the traversal's box tests
and the BVH quantiser call fma explicitly), so the integrator's float arithmetic rounds as the
reference's host build does (measured cost on the stress-scene render: 1.5 %).  The host loader
is compiled with `-ffp-contract=off` for the same reason, on every CPU (x86-64 and aarch64).
Translation units compile in parallel; no cmake.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "liblts_gb300.so")
APP = os.path.join(LIBDIR, "lts_render_app")  # the C host program (host/render_app.c)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Extra nvcc arguments for tuning builds (e.g. LTS_NVCC_EXTRA="-DLTS_TRACE_MIN_BLOCKS=5"); pass
# force=True (or delete _lib/obj) when changing them.
EXTRA = os.environ.get("LTS_NVCC_EXTRA", "").split()


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    nvcc = _nvcc()
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    cu, cpp = _sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "lts_capi.h"))
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(LIBDIR, "obj", f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, os.path.abspath(__file__)] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler",
                         "-fPIC,-ffp-contract=off", "-Xptxas", "-warn-spills", *EXTRA, "-c", src, "-o", obj])
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(LIBDIR, "obj", f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"compile failed: {cmd[-3]}")
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart", "-Xcompiler", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(LIB + ".tmp", LIB)
    app_src = os.path.join(HERE, "host", "render_app.c")
    if os.path.exists(app_src) and (force or _stale(APP, [app_src, LIB, os.path.join(HERE, "..", "include", "lts_capi.h")])):
        # the thin C host program over the C-ABI, linked against the library in place
        cmd = ["gcc", "-O2", "-std=c99", "-Wall", "-o", APP + ".tmp", app_src, "-L" + LIBDIR, "-llts_gb300",
               "-Wl,-rpath," + LIBDIR]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("host program link failed")
        os.replace(APP + ".tmp", APP)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
