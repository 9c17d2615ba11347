"""Build of the in-tree CUDA library libcovgpu.so (sm_103a only).

Each translation unit under csrc/ is compiled by its own nvcc process, in
parallel, with one -gencode for sm_103a; the objects are linked into
coldcase_gb300/_lib/libcovgpu.so.  A unit is recompiled only when its source
or a header it includes is newer than its object.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIBNAME = "libcovgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
           "--expt-relaxed-constexpr"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcovgpu.so")


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(obj, src, hdr_mtime):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or hdr_mtime > t


def build(verbose=False, force=False, extra_flags=()):
    """Compile every csrc/*.cu for sm_103a and link libcovgpu.so; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(OBJDIR, exist_ok=True)
    hdr_mtime = max([0.0] + [os.path.getmtime(h) for h in _headers()])
    jobs = []
    objs = []
    for src in _sources():
        obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, src, hdr_mtime):
            cmd = [nvcc] + ARCH + NVFLAGS + list(extra_flags) + ["-I", INCLUDE, "-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
        if verbose and (p.stdout or p.stderr):
            print(p.stdout + p.stderr)
        return cmd

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(run, jobs))
    out = lib_path()
    if jobs or not os.path.exists(out):
        tmp = out + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
        os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
