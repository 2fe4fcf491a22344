#!/usr/bin/env python3
"""Build OpenMBIR-TEM's own reconstruction programs from their sources into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  The two command-line programs HAADFReconstruction and
BFReconstruction (Code/Applications/*) and the library they drive (Code/MBIRLib, the POSIX
part of Code/MXA) are compiled where they lie in the reference tree, unmodified, with g++.
Only two things stand in for the reference's build system and its external libraries:

* oracle/ref_shim/ -- headers cmake would generate (MBIRLib/MBIRLib.h, MXA/MXA.h, version),
  and minimal Boost (shared_ptr, shared_array, mt19937, uniform_int, variate_generator) and
  TBB (task, task_list, task_group, task_scheduler_init) stand-ins written for this recipe;
* oracle/ref_shim/ref_runtime.cpp -- a fixed-seed switch for the reference's clock seeds and a
  zeroing operator new (the engines leave some parameter fields unset).

A third program, SigmaXEstimate (oracle/ref_shim/ref_sigmax_main.cpp, a main of this recipe),
drives the reference's SigmaXEstimation filter the way its GUIs do.  The objects and the
programs go to oracle/_ref/ (git-ignored).  They are the parity pin of
the CPU restatement oracle/mbir_oracle.c: tests/test_oracle_vs_ref.py runs both on the same
inputs and compares their outputs, and tests/golden/make_golden.py stores small outputs of the
programs as fixtures so that the pin also holds where the reference tree is absent.

Usage: python oracle/build_ref.py [--reference DIR] [--jobs N]
Exit status 0 when both programs were built (or are up to date), 1 when the reference tree is
absent or a compile failed (the log names the file).
"""
import argparse
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim")
DEFAULT_REFERENCE = "/root/reference"

# Translation units of MBIRLib (Code/MBIRLib/*/SourceList.cmake; the *_Extra.cpp and
# *_UpdateVoxels.cpp files are included by their engine .cpp there, HEADER_FILE_ONLY).
MBIRLIB_SOURCES = [
    "BrightField/BFForwardModel.cpp",
    "BrightField/BFForwardProject.cpp",
    "BrightField/BF_QGGMRFPriorModel.cpp",
    "BrightField/BFUpdateYSlice.cpp",
    "BrightField/BFReconstructionEngine.cpp",
    "BrightField/BFMultiResolutionReconstruction.cpp",
    "Common/allocate.c",
    "Common/AMatrixCol.cpp",
    "Common/EIMTime.c",
    "Common/EIMImage.cpp",
    "Common/AbstractFilter.cpp",
    "Common/FilterPipeline.cpp",
    "Common/Observer.cpp",
    "Common/Observable.cpp",
    "Common/VoxelUpdateList.cpp",
    "GenericFilters/BackgroundCalculation.cpp",
    "GenericFilters/CalculateAMatrixColumn.cpp",
    "GenericFilters/ComputeInitialOffsets.cpp",
    "GenericFilters/CostData.cpp",
    "GenericFilters/DetectorParameters.cpp",
    "GenericFilters/DetectorResponse.cpp",
    "GenericFilters/InitialReconstructionBinReader.cpp",
    "GenericFilters/InitialReconstructionInitializer.cpp",
    "GenericFilters/MRCSinogramInitializer.cpp",
    "GenericFilters/RawSinogramInitializer.cpp",
    "GenericFilters/SigmaXEstimation.cpp",
    "GenericFilters/TomoFilter.cpp",
    "HAADF/HAADF_QGGMRFPriorModel.cpp",
    "HAADF/HAADF_MultiResolutionReconstruction.cpp",
    "HAADF/HAADF_ForwardModel.cpp",
    "HAADF/HAADF_ForwardProject.cpp",
    "HAADF/HAADF_ReconstructionEngine.cpp",
    "IOFilters/AvizoUniformCoordinateWriter.cpp",
    "IOFilters/DetectorResponseWriter.cpp",
    "IOFilters/GainsOffsetsReader.cpp",
    "IOFilters/RawGeometryWriter.cpp",
    "IOFilters/MRCReader.cpp",
    "IOFilters/MRCWriter.cpp",
    "IOFilters/NuisanceParamWriter.cpp",
    "IOFilters/NuisanceParamReader.cpp",
    "IOFilters/SinogramBinWriter.cpp",
    "Reconstruction/ReconstructionInputs.cpp",
    "Reconstruction/QGGMRF_Functions.cpp",
]
# Code/MXA/Common/SourceList.cmake and Utilities/SourceList.cmake, POSIX part.
MXA_SOURCES = [
    "Common/IO/Private/MXAPrivateFileReader.cpp",
    "Common/IO/Private/MXAPrivateFileWriter.cpp",
    "Utilities/MXADir.cpp",
    "Utilities/MXAFileInfo.cpp",
    "Utilities/MD5.cpp",
]
PROGRAMS = {
    "HAADFReconstruction": ["main.cpp", "HAADFReconstructionArgsParser.cpp"],
    "BFReconstruction": ["main.cpp", "BFReconstructionArgsParser.cpp"],
}
# harnesses of this recipe (oracle/ref_shim) over reference classes the programs do not reach
HARNESSES = {"SigmaXEstimate": "ref_sigmax_main.cpp"}

# -O2 as the reference's release build; no FMA contraction so that its FP64 arithmetic rounds
# operation by operation (as the oracle's does) on hosts whose default ISA has FMA.
COMMON_FLAGS = ["-O2", "-fno-strict-aliasing", "-ffp-contract=off", "-w", "-pthread",
                "-DOpenMBIR_USE_PARALLEL_ALGORITHMS=1"]


def _obj_name(rel):
    return rel.replace("/", "__").rsplit(".", 1)[0] + ".o"


def _compile(src, obj, includes, extra):
    is_c = src.endswith(".c")
    cmd = (["gcc", "-std=gnu99"] if is_c else ["g++", "-std=gnu++14"]) + COMMON_FLAGS + extra
    cmd += [f"-I{d}" for d in includes] + ["-c", src, "-o", obj]
    if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src):
        return None
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return f"{src}:\n{r.stderr[-4000:]}"
    return None


def build(reference=DEFAULT_REFERENCE, jobs=None, quiet=False):
    """Compile both programs into oracle/_ref; returns True on success."""
    code = os.path.join(reference, "Code")
    if not os.path.isdir(os.path.join(code, "MBIRLib")):
        if not quiet:
            print(f"build_ref: reference tree not found under {reference}", file=sys.stderr)
        return False
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    includes = [SHIM, code, os.path.join(code, "MBIRLib"), os.path.join(code, "MXA")]
    units = []
    for rel in MBIRLIB_SOURCES:
        extra = []
        if rel == "Common/EIMTime.c":
            extra = ["-DEIMTOMO_getMilliSeconds=ref_clock_ms"]
        units.append((os.path.join(code, "MBIRLib", rel), "MBIRLib__" + _obj_name(rel), extra))
    for rel in MXA_SOURCES:
        units.append((os.path.join(code, "MXA", rel), "MXA__" + _obj_name(rel), []))
    units.append((os.path.join(SHIM, "ref_runtime.cpp"), "shim__ref_runtime.o", []))
    for prog, src in HARNESSES.items():
        units.append((os.path.join(SHIM, src), prog + "__" + _obj_name(src), []))
    for prog, files in PROGRAMS.items():
        for f in files:
            rel = os.path.join("Applications", prog, f)
            units.append((os.path.join(code, rel), prog + "__" + _obj_name(f), []))
    objs = {}
    errors = []
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        futs = {}
        for src, name, extra in units:
            obj = os.path.join(OUT, "obj", name)
            objs[name] = obj
            futs[ex.submit(_compile, src, obj, includes, extra)] = src
        for fu in cf.as_completed(futs):
            err = fu.result()
            if err:
                errors.append(err)
    if errors:
        print("build_ref: compile errors\n" + "\n".join(errors), file=sys.stderr)
        return False
    lib_objs = [o for n, o in objs.items() if n.startswith(("MBIRLib__", "MXA__", "shim__"))]
    for prog in list(PROGRAMS) + list(HARNESSES):
        exe = os.path.join(OUT, prog)
        pobjs = [o for n, o in objs.items() if n.startswith(prog + "__")]
        newest = max(os.path.getmtime(o) for o in lib_objs + pobjs)
        if os.path.exists(exe) and os.path.getmtime(exe) >= newest:
            continue
        cmd = ["g++", "-pthread", "-o", exe] + pobjs + lib_objs + ["-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(f"build_ref: link of {prog} failed\n{r.stderr[-4000:]}", file=sys.stderr)
            return False
    if not quiet:
        print(f"build_ref: {', '.join(list(PROGRAMS) + list(HARNESSES))} in {OUT}")
    return True


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    ap.add_argument("--jobs", type=int, default=None)
    a = ap.parse_args()
    return 0 if build(a.reference, a.jobs) else 1


if __name__ == "__main__":
    sys.exit(main())
