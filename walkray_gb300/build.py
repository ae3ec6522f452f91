"""Build recipe for the in-tree CUDA library (libwalkray_gpu.so, sm_103a) and
the oracle programs.

    python -m walkray_gb300.build            # library + oracle
    python -m walkray_gb300.build --lib      # library only

Every translation unit is compiled by nvcc in parallel, with IEEE division
and square root.  The traversal code whose results must equal the
reference's FP32 bit for bit (box face test, triangle test, face normals,
NoSelfCondition) spells every product and sum as an unfused round-to-nearest
intrinsic (wr_device.cuh: add_x, mul_x, ...), which no compiler setting
contracts, so the path tracer's translation units are compiled with
contraction into fused multiply-adds (-fmad=true).  The bidirectional /
VCM / photon-mapping unit (bpt.cu) is not: its estimators keep or drop
merges and photons by the last bit of hit points against the light points'
bounding box and the hash grid, as the reference's unfused FP32 does, and
contraction moved those decisions far enough to shift its images off the
reference's (measured: photon mapping on the Cornell box 4 % brighter).
Host code uses -ffp-contract=off, on x86-64 and aarch64 alike.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwalkray_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNFUSED = {"bpt.cu"}  # translation units compiled without contraction (see the module docstring)


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src: str, nvcc: str) -> str:
    out = os.path.join(OBJ, src.rsplit(".", 1)[0] + ".o")
    path = os.path.join(CSRC, src)
    host = "-Xcompiler=-fPIC,-fopenmp,-ffp-contract=off,-O3"
    if src.endswith(".cu"):
        fmad = "-fmad=false" if src in UNFUSED else "-fmad=true"
        cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", fmad, "-prec-div=true", "-prec-sqrt=true",
               host, "-c", path, "-o", out]
    else:
        cmd = [nvcc, "-std=c++17", "-O3", host, "-c", path, "-o", out]
    # an object is current when it is newer than its sources and was built by the same command
    stamp = out + ".cmd"
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "walkray.h"))
    if (os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps)
            and os.path.exists(stamp) and open(stamp).read() == " ".join(cmd)):
        return out
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(" ".join(cmd))
    return out


def build_lib(verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler=-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def reference_dir() -> str:
    """The WalkRay source tree the oracle's reference harness compiles: the
    environment variable WR_REFERENCE_DIR, else the oracle Makefile's default
    when that tree is present; "" when there is none (as on a machine that
    only runs the prebuilt library)."""
    ref = os.environ.get("WR_REFERENCE_DIR", "")
    if not ref:
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref-dir"],
                           capture_output=True, text=True)
        ref = r.stdout.strip() if r.returncode == 0 else ""
    return ref if ref and os.path.isfile(os.path.join(ref, "kdtree.cpp")) else ""


def build_oracle(verbose: bool = False) -> None:
    """The C restatement always; the reference harness too when a WalkRay
    source tree is present (reference_dir)."""
    odir = os.path.join(ROOT, "oracle")
    r = subprocess.run(["make", "-s", "-C", odir, "port"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    ref = reference_dir()
    if ref:
        r = subprocess.run(["make", "-s", "-j8", "-C", odir, "ref", f"REF={ref}"], capture_output=True, text=True)
        if r.returncode != 0 and verbose:
            print("reference harness not built:", r.stderr[-2000:])
    if verbose:
        print("built oracle")


if __name__ == "__main__":
    build_lib(verbose=True)
    if "--lib" not in sys.argv:
        build_oracle(verbose=True)
