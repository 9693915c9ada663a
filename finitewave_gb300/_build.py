"""Compile the CUDA sources of finitewave_gb300 into libfwgpu.so (sm_103a).

The library is built in-tree into ``finitewave_gb300/_lib/`` with nvcc: each
translation unit is compiled in parallel, then linked into one shared object
that exports the C ABI declared in ``include/fwgpu.h``.  Translation units
that must reproduce the reference's float64 arithmetic bit for bit are
compiled with ``--fmad=false`` (no fused multiply-add contraction).
"""
import concurrent.futures
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "_lib")
BUILDDIR = os.path.join(PKG, "_lib", "_build")
LIBNAME = "libfwgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-fvisibility=hidden", "-I" + INCLUDE, "-I" + CSRC,
          "--expt-relaxed-constexpr"]
# translation unit -> extra flags
UNITS = {
    "fw_capi.cu": [],
    "fw_weights.cu": ["--fmad=false"],
    "fw_step.cu": ["--fmad=false"],
    "fw_fused.cu": [],
    "fw_batch.cu": ["--prec-div=false", "--ftz=true"],
    "fw_fused_ap.cu": ["--prec-div=false", "--ftz=true"],
    "fw_fused_ms.cu": ["--prec-div=false", "--ftz=true"],
    "fw_fused_fk.cu": ["--prec-div=false", "--ftz=true"],
    "fw_fused_bk.cu": ["--prec-div=false", "--ftz=true"],
    "fw_step_detailed_tp06_f64.cu": ["--fmad=false"],
    "fw_step_detailed_tp06_f32.cu": ["--prec-div=false", "--prec-sqrt=false",
                                     "--ftz=true"],
    "fw_step_detailed_crn_f64.cu": ["--fmad=false"],
    "fw_step_detailed_crn_f32.cu": ["--prec-div=false", "--prec-sqrt=false",
                                    "--ftz=true"],
    "fw_step_detailed_lr91_f64.cu": ["--fmad=false"],
    "fw_step_detailed_lr91_f32.cu": ["--prec-div=false", "--prec-sqrt=false",
                                     "--ftz=true"],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to "
                       "build finitewave_gb300")


def _sources_digest():
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for f in sorted(os.listdir(d)):
            if f.endswith((".cu", ".cuh", ".h")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(f.encode() + fh.read())
    h.update(repr((ARCH, COMMON, UNITS)).encode())
    return h.hexdigest()


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def build(force=False, verbose=False):
    """Build libfwgpu.so if missing or stale; return its path."""
    os.makedirs(BUILDDIR, exist_ok=True)
    digest = _sources_digest()
    stamp = os.path.join(LIBDIR, "build.stamp")
    out = lib_path()
    if (not force and os.path.exists(out) and os.path.exists(stamp)
            and open(stamp).read() == digest):
        return out
    exe = nvcc()

    def compile_one(unit):
        obj = os.path.join(BUILDDIR, unit.replace(".cu", ".o"))
        cmd = [exe] + ARCH + COMMON + UNITS[unit] + [
            "-c", os.path.join(CSRC, unit), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, flush=True)
        return obj

    with concurrent.futures.ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_one, sorted(UNITS)))
    tmp = out + ".tmp%d" % os.getpid()
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, out)
    with open(stamp, "w") as f:
        f.write(digest)
    return out


if __name__ == "__main__":
    print(build(force=True, verbose=True))
