"""Build libmbir_gb300.so (sm_103a) in-tree with nvcc; no cmake, no torch extension.

    python openmbir-tem_gb300/build.py            # build if sources are newer than the .so
    python openmbir-tem_gb300/build.py --force

Translation units compile in parallel; the shared library lands next to this file.
"""
import argparse
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmbir_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["mbir_sweep_f32.cu", "mbir_sweep_f32_bf.cu", "mbir_sweep_f32_hbm.cu",
           "mbir_sweep_f32_hbm_bf.cu",
           "mbir_sweep_f32_batch3.cu", "mbir_sweep_f32_batch5.cu", "mbir_sweep_f64.cu",
           "mbir_kernels.cu", "mbir_bfassist.cu",
           "mbir_exact.cu", "mbir_bf.cu", "mbir_noalloc.cu",
           "mbir_engine.cu", "mbir_engine_bf.cu", "mbir_shard.cu", "mbir_batch.cu", "mbir_server.cpp", "mrc_io.cpp",
           "mbir_schedule.cpp", "mbir_colour.cu", "mbir_capi.cpp"]
HEADERS = ["mbir_internal.h", "mbir_engine.h", "mbir_sweep.cuh", "mbir_batch.h",
           "mbir_server.h", "mbir_schedule.h"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    raise RuntimeError("nvcc not found")


def _stale():
    if not os.path.exists(LIB):
        return True
    if any(not os.path.exists(os.path.join(HERE, "bin", n))
           for n in ("HAADFReconstruction", "BFReconstruction")):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    deps.append(os.path.join(ROOT, "include", "mbir_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose=False, ptxas_v=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, src),
           "-o", obj]
    # host arithmetic must not be contracted into FMAs (the FP64 tables and per-view solves
    # are compared bit for bit with the oracle on every host architecture)
    cmd[1:1] = ["-Xcompiler", "-ffp-contract=off"]
    if src.endswith(".cu"):
        cmd[1:1] = ARCH + ["-lineinfo", "--expt-relaxed-constexpr"]
        # no fused multiply-adds: the reference-exact and BF passes must reproduce FP64 operation
        # by operation, and every FP32 sweep kernel (single slice, batched, any caller) must round
        # identically so a reconstruction gives the same bits alone and inside a batch
        if src in ("mbir_exact.cu", "mbir_bf.cu") or src.startswith("mbir_sweep_f32"):
            cmd[1:1] = ["-fmad=false"]
        if ptxas_v:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd[1:1] = ["-x", "c++"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose=False, ptxas_v=False):
    """Compile the CUDA engine into openmbir-tem_gb300/libmbir_gb300.so; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, ptxas_v), SOURCES))
    objs = [o for o, _ in results]
    if ptxas_v:
        for _, log in results:
            if log:
                print(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl",
                                                             "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli(verbose)
    return LIB


CLI_SRC = os.path.join(HERE, "cli", "mbir_reconstruct.cpp")
BIN = os.path.join(HERE, "bin")
CLI_PROGRAMS = {"HAADFReconstruction": 0, "BFReconstruction": 1}


def build_cli(verbose=False):
    """The two command-line programs (bin/HAADFReconstruction, bin/BFReconstruction) over the
    C++ pipeline classes of include/mbir_gb300.hpp, linked to libmbir_gb300.so next to them
    (rpath $ORIGIN/..)."""
    os.makedirs(BIN, exist_ok=True)
    for name, bf in CLI_PROGRAMS.items():
        exe = os.path.join(BIN, name)
        deps = [CLI_SRC, LIB, os.path.join(ROOT, "include", "mbir_gb300.h"),
                os.path.join(ROOT, "include", "mbir_gb300.hpp")]
        if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(d) for d in deps):
            continue
        cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-pthread", f"-DMBIR_CLI_BF={bf}", "-o", exe,
               CLI_SRC,
               f"-L{HERE}", "-l:libmbir_gb300.so", "-Wl,-rpath,$ORIGIN/.."]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed for {name}:\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-v", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force or a.ptxas_v, verbose=a.verbose, ptxas_v=a.ptxas_v))
    sys.exit(0)
