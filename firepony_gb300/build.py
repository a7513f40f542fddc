"""In-tree build of the native libraries.

* ``libfpengine.so`` — the CUDA engine and its C ABI (``include/firepony_gb300.h``, and the reference store of
  ``include/firepony_gb300_store.h``), compiled by nvcc for sm_103a only.
* ``libfpsynth.so`` — the seeded synthetic-input generator (host C++).

Everything is compiled in parallel into ``firepony_gb300/_build`` (git-ignored). Sources are rebuilt when
they are newer than their outputs.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation units of the engine: (source, extra nvcc flags)
ENGINE_UNITS = [
    ("engine.cu", []),
    ("k_prep.cu", []),
    ("k_baq64.cu", ["-fmad=false"]),   # FP64 HMM: bit-exact replay of the reference's operation order
    ("k_baq_tpr.cu", []),
    ("k_baq_seg.cu", []),               # band class 0 FP32 (checkpointed forward rows, packed pairs)
    ("k_baq_exact.cu", ["-fmad=false"]),  # exact FP64 replay (explicit rounding intrinsics throughout)
    ("k_baq_wide.cu", []),              # FP32 certified HMM for bands wider than 15
    ("k_covariates.cu", []),
    ("k_sort.cu", []),
    ("k_post.cu", ["-fmad=false"]),    # empirical quality: exact IEEE double sums and products
    ("k_precision.cu", []),             # precision trace: FP32 vs FP64 MAP quality per read
    ("k_probe.cu", []),                 # FP32 SIMT throughput probe (roofline denominator)
    ("report.cpp", []),
    ("refstore.cu", []),                # reference store: shared-memory segments, one device copy per GPU
]


def _newer(src: list[Path], out: Path) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in src)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _headers() -> list[Path]:
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))


def build_engine(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libfpengine.so"
    hdrs = _headers()
    objs = []
    jobs = []
    for src, extra in ENGINE_UNITS:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if _newer([s] + hdrs, o):
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
                   "-I", str(INCLUDE), "-I", str(CSRC), *extra, "-c", str(s), "-o", str(o)]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    if jobs or _newer(objs, out):
        _run([NVCC, *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcudart"])
    return out


def build_synth() -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libfpsynth.so"
    src = CSRC / "synth.cpp"
    if _newer([src], out):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-o", str(out), str(src)])
    return out


CUDA_HOME = Path(NVCC).resolve().parent.parent


def zlib_available() -> bool:
    return any(Path(d, "zlib.h").exists() for d in ("/usr/include", "/usr/local/include"))


def build_bam() -> Path | None:
    """libfpbam.so: BGZF/BAM decoding into the engine's batch layout (include/firepony_gb300_bam.h). Needs
    zlib; skipped (None) where its header is absent."""
    if not zlib_available():
        return None
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libfpbam.so"
    hdrs = [INCLUDE / "firepony_gb300_bam.h", INCLUDE / "firepony_gb300.h", CSRC / "bam_internal.h",
            CSRC / "bgzf_inflate.cuh"]
    host_src, host_obj = CSRC / "bam.cpp", BUILD / "bam.cpp.o"
    gpu_src, gpu_obj = CSRC / "bam_gpu.cu", BUILD / "bam_gpu.cu.o"
    jobs = []
    if _newer([host_src] + hdrs, host_obj):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-I", str(INCLUDE), "-I", str(CSRC),
                     "-I", str(CUDA_HOME / "include"), "-c", str(host_src), "-o", str(host_obj)])
    if _newer([gpu_src] + hdrs, gpu_obj):
        jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", str(INCLUDE),
                     "-I", str(CSRC), "-c", str(gpu_src), "-o", str(gpu_obj)])
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, jobs))
    if jobs or _newer([host_obj, gpu_obj], out):
        _run([NVCC, *ARCH, "-shared", "-o", str(out), str(host_obj), str(gpu_obj), "-Xcompiler", "-pthread",
              "-lcudart", "-lz"])
    return out


def build_inflate_check(sanitize: bool = True) -> Path:
    """Host build of the BGZF block decoder's unit check (tests/native/inflate_check.cpp) against zlib, with the
    address and undefined-behaviour sanitizers."""
    BUILD.mkdir(exist_ok=True)
    out = BUILD / ("inflate_check_san" if sanitize else "inflate_check")
    src = ROOT / "tests" / "native" / "inflate_check.cpp"
    if _newer([src, CSRC / "bgzf_inflate.cuh"], out):
        san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined", "-g"] if sanitize else []
        _run(["g++", "-O1", "-std=c++17", *san, "-I", str(CSRC), "-o", str(out), str(src), "-lz"])
    return out


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        fs = [ex.submit(build_engine, verbose), ex.submit(build_synth), ex.submit(build_bam)]
        for f in fs:
            f.result()


if __name__ == "__main__":
    build_all(verbose=bool(os.environ.get("FP_VERBOSE")))
    print("built", *sorted(p.name for p in BUILD.glob("*.so")))
