"""Builds the engine's shared library in-tree: voro_gb300/_lib/libvorogpu.so.

nvcc compiles each CUDA translation unit for sm_103a in parallel and links a
plain C-ABI shared library (no torch types, no Python objects).
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libvorogpu.so")
CLI = os.path.join(LIBDIR, "voro++")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["vgpu_api.cu", "vgpu_bin.cu", "vgpu_sort.cu", "vgpu_cell.cu", "vgpu_clip_mixed.cu", "vgpu_clip_fp64.cu",
           "vgpu_finish.cu", "vgpu_noalloc.cu", "vgpu_locate.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wno-deprecated-declarations",
              "-diag-suppress", "1444"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the engine cannot be built")
    return cand


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith((".h", ".hh"))]
    files += [os.path.join(HERE, "cli", f) for f in os.listdir(os.path.join(HERE, "cli")) if f.endswith(".cc")]
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(CLI):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags=None, out=None) -> str:
    """Compiles the library if a source is newer than it; returns its path.
    ``out`` writes a variant library elsewhere (e.g. with other -D flags)."""
    target = out or LIB
    if out is None and not force and up_to_date():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tag = "" if out is None else "_" + str(abs(hash(out)) % 100000)
    nvcc = _nvcc()
    flags = NVCC_FLAGS + list(extra_flags or [])
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(LIBDIR, src.replace(".cu", tag + ".o"))
        cmd = [nvcc] + ARCH + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(obj)
    errors = []
    for (src, p), obj in zip(procs, objs):
        log, _ = p.communicate()
        if verbose and log:
            print(log)
        if p.returncode != 0:
            # nvcc has crashed (SIGSEGV) on aarch64 hosts, not reproducibly: retry
            # serially, again, then without line tables, and last with a lower
            # ptxas optimisation level
            ok = False
            nolines = [f for f in flags if f != "-lineinfo"]
            for fl in (flags, flags, nolines, nolines + ["-Xptxas", "-O2"]):
                cmd = [nvcc] + ARCH + fl + ["-c", os.path.join(CSRC, src), "-o", obj]
                r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
                if r.returncode == 0:
                    ok = True
                    break
                log = r.stdout
            if not ok:
                errors.append(f"{src}:\n{log}")
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = target + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout)
    os.replace(tmp, target)
    for o in objs:
        try:
            os.remove(o)
        except OSError:
            pass
    if out is None:
        build_cli()
    return target


def build_cli() -> str:
    """The command-line utility (voro_gb300/cli/voro++.cc, the reference's
    voro++ on this engine): a host program over include/voro_gb300.hh, linked
    against libvorogpu.so beside it."""
    cxx = shutil.which("g++") or "g++"
    src = os.path.join(HERE, "cli", "voro++.cc")
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-I", INCLUDE, src, "-L", LIBDIR, "-lvorogpu",
                        "-Wl,-rpath,$ORIGIN", "-o", CLI + ".tmp"], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("voro++ build failed:\n" + r.stdout)
    os.replace(CLI + ".tmp", CLI)
    return CLI


if __name__ == "__main__":
    print(build(force=True, verbose=True))
