"""Builds libdpstokes_gb300.so in-tree (doublyperiodicstokes_gb300/lib/) with
nvcc for sm_103a: each translation unit is compiled in parallel, then linked
with cuFFT.  No CMake, no setuptools; the recipe is the same on x86 build
hosts and on the aarch64 GPU hosts.

    python -m doublyperiodicstokes_gb300.build [--force] [--verbose]
"""
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIBNAME = "libdpstokes_gb300.so"
SOURCES = ["dpst_engine.cu", "dpst_particles.cu", "dpst_kspace.cu", "dpst_bvp.cu", "dpst_adjoint.cu",
           "dpst_grad.cu", "dpst_batch.cu", "dpst_ztc.cu", "dpst_tp.cu", "dpst_bvp_df.cu",
           "dpst_fft.cu", "dpst_fft_df.cu"]
HEADERS = ["dpst_internal.cuh", "dpst_kdev.cuh", "dpst_pdev.cuh", "dpst_host.cuh", "dpst_launch.cuh",
           "dpst_df64.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + os.path.join(ROOT, "include")]


def nvcc_path():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _digest():
    h = hashlib.sha256()
    for f in SOURCES + HEADERS:
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(f.encode() + fh.read())
    with open(os.path.join(ROOT, "include", "dpstokes_gb300.h"), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile and link the library if its sources changed; return its path."""
    os.makedirs(LIBDIR, exist_ok=True)
    stamp = os.path.join(LIBDIR, "build.stamp")
    digest = _digest()
    out = lib_path()
    if not force and os.path.exists(out) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return out
    nvcc = nvcc_path()
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(LIBDIR, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, pr in procs:
        outp, _ = pr.communicate()
        if pr.returncode != 0:
            failed.append((cmd, outp.decode(errors="replace")))
        elif verbose and outp:
            print(outp.decode(errors="replace"))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = out + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcufft"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, out)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
