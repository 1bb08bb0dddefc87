"""Build the sm_103a C-ABI library ``libcato_gpu.so`` in-tree (``fvleg_2d_gb300/_lib/``).

The stage kernel family is instantiated once per (precision, flux) pair from ``stage_inst.cu``
(the double-float ones once per reconstruction and kernel kind) so that the units compile in
parallel; the FP64 units and the helper kernels are built
with ``--fmad=false`` (each reference operation rounds on its own), the FP32 mixed units with
FMA contraction, fast square root and flush-to-zero, the double-float units with FMA contraction
and IEEE FP32 semantics (their pair arithmetic is written with explicitly rounded intrinsics).
No CMake, no torch: nvcc and a C++ host compiler only.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libcato_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
N_FLUX = 9


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcato_gpu.so")


def _sources_digest(extra: list[str]) -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            if name.endswith((".cu", ".cuh", ".h", ".hpp", ".cpp")):
                with open(os.path.join(d, name), "rb") as f:
                    h.update(name.encode())
                    h.update(f.read())
    h.update(" ".join(extra).encode())
    return h.hexdigest()


def _units() -> list[tuple[str, list[str]]]:
    common = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", INCLUDE]
    # developer knob: extra nvcc flags for every unit (e.g. -DCATO_DF_MIN_BLOCKS=2)
    common += os.environ.get("CATO_NVCC_FLAGS", "").split()
    units = []
    src = os.path.join(CSRC, "stage_inst.cu")
    for real, flags in (("double", ["--fmad=false"]),
                        ("float", ["--fmad=true", "-prec-sqrt=false", "-ftz=true"]),
                        ("df", ["--fmad=true"])):
        for flux in range(N_FLUX):
            # the double-float kernels take ~10x longer in ptxas: one unit per reconstruction
            # and kernel kind keeps every unit under a minute
            parts = ([(rc, part) for rc in (0, 3, 5) for part in (1, 2)] if real == "df"
                     else [(None, 0)])
            for rc, part in parts:
                tag = f"stage_{real}_{flux}" + ("" if rc is None else f"_r{rc}_k{part}")
                obj = os.path.join(BUILD_DIR, tag + ".o")
                defs = [f"-DCATO_REAL={real}", f"-DCATO_FLUX={flux}"]
                if rc is not None:
                    defs += [f"-DCATO_RECON={rc}", f"-DCATO_PART={part}"]
                cmd = [nvcc(), *ARCH, *common, *flags, *defs, "-c", src, "-o", obj]
                units.append((obj, cmd))
    # longest first, so that the slow double-float units start before the rest
    units.sort(key=lambda u: 0 if "-DCATO_REAL=df" in u[1] else 1)
    for src in ("cato_capi.cu", "cato_batch.cu", "cato_noalloc.cu", "cato_pbc.cu"):
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        units.append((obj, [nvcc(), *ARCH, *common, "--fmad=false", "-c", path, "-o", obj]))
    return units


def lib_path() -> str:
    return os.path.join(OUT_DIR, LIB_NAME)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile (if sources changed) and return the path of libcato_gpu.so."""
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    units = _units()
    digest = _sources_digest([u[1][-1] for u in units] + [" ".join(units[0][1])])
    stamp = os.path.join(BUILD_DIR, "stamp")
    out = lib_path()
    if os.path.exists(out) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return out
    jobs = jobs or max(1, min(len(units), os.cpu_count() or 4))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)

    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(run, [u[1] for u in units]))
    tmp = out + ".tmp"
    run([nvcc(), *ARCH, "-shared", "-o", tmp, *[u[0] for u in units], "-lcudart"])
    os.replace(tmp, out)
    with open(stamp, "w") as f:
        f.write(digest)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
