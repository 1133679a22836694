"""Build the engine's shared library for sm_103a, in-tree.

    python -m thoth_gb300.build             # -> thoth_gb300/_build/libthoth_gpu.so
    python -m thoth_gb300.build --sanitize  # -> thoth_gb300/_build_san/libthoth_gpu.so, host
                                            #    code under AddressSanitizer and UBSan

nvcc cross-compiles without a GPU. The Joe-Kuo table is embedded into the
library from thoth_gb300/data/joe_kuo_6_21201.bin through a generated C file.
"""
import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
BUILD_SAN = HERE / "_build_san"
CSRC = HERE / "csrc"
LIB = BUILD / "libthoth_gpu.so"
# host code of the sanitized build (nvcc splits -Xcompiler values at commas: one flag each)
SAN_HOST = ["-fsanitize=address", "-fsanitize=undefined", "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["book_batch.cu", "book_heston.cu", "book_multi.cu", "book_lsv.cu", "book_gbm.cu", "kernels.cu", "thoth_gpu.cu",
           "surrogate.cu", "surrogate_host.cu", "greeks.cu", "american.cu", "american_host.cu", "calib.cu"]
# the path kernels flush FP32 denormals: no value on the path is subnormal, and
# without it every MUFU approximation (rcp, rsqrt, lg2, ex2) carries a
# denormal fix-up sequence (11 % of the Heston step's time)
FLAGS = {"kernels.cu": ["-ftz=true"], "book_batch.cu": ["-ftz=true"], "book_gbm.cu": ["-ftz=true"], "book_heston.cu": ["-ftz=true"],
         "book_lsv.cu": ["-ftz=true"], "book_multi.cu": ["-ftz=true"],
         # the exercise tables and the regression solve are compared bit for bit with the
         # oracle: no contraction of a * b + c into a fused multiply-add on the host
         "american_host.cu": ["-Xcompiler", "-ffp-contract=off"],
         "thoth_gpu.cu": ["-Xcompiler", "-ffp-contract=off"],
         # the calibration ensemble rounds every expression as the reference does
         "calib.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _gen_blob():
    data = (HERE / "data" / "joe_kuo_6_21201.bin").read_bytes()
    out = BUILD / "jk_blob.c"
    lines = ["#include <stddef.h>", "const unsigned char thoth_jk_blob[] = {"]
    for i in range(0, len(data), 32):
        lines.append(",".join(str(b) for b in data[i:i + 32]) + ",")
    lines.append("};")
    lines.append("const size_t thoth_jk_blob_size = %d;" % len(data))
    text = "\n".join(lines) + "\n"
    if not out.exists() or out.read_text() != text:
        out.write_text(text)
    return out


def _xc(flags):
    return [x for f in flags for x in ("-Xcompiler", f)]


def _compile(src, verbose, out=BUILD, sanitize=False):
    obj = out / (pathlib.Path(src).stem + ".o")
    cmd = [nvcc(), "-c", str(CSRC / src), "-o", str(obj), "-O1" if sanitize else "-O3", "-lineinfo", "-std=c++17",
           "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"), "-I", str(CSRC)] + ARCH + FLAGS.get(src, [])
    if sanitize:
        cmd += ["-g"] + _xc(SAN_HOST)
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr))
    return obj, r.stderr


def build_sanitized(out=BUILD_SAN):
    """The library with its host code under AddressSanitizer and UBSan, in `out` (the
    device code is the same). A process loads it with THOTH_GPU_LIB pointing at it and the
    sanitizer runtimes preloaded (LD_PRELOAD)."""
    out = pathlib.Path(out)
    out.mkdir(parents=True, exist_ok=True)
    BUILD.mkdir(exist_ok=True)
    blob = _gen_blob()
    blob_o = out / "jk_blob.o"
    subprocess.run(["gcc", "-c", "-fPIC", "-O1", str(blob), "-o", str(blob_o)], check=True)
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = [r[0] for r in ex.map(lambda s: _compile(s, False, out, True), SOURCES)]
    lib = out / LIB.name
    tmp = out / (LIB.name + ".tmp")
    cmd = [nvcc(), "-shared", "-o", str(tmp)] + [str(o) for o in objs] + [str(blob_o)] + ARCH + ["-lcudart"]
    subprocess.run(cmd + _xc(SAN_HOST[:2]), check=True)
    os.replace(tmp, lib)
    return lib


def build(verbose=False):
    BUILD.mkdir(exist_ok=True)
    blob = _gen_blob()
    blob_o = BUILD / "jk_blob.o"
    subprocess.run(["gcc", "-c", "-fPIC", "-O1", str(blob), "-o", str(blob_o)], check=True)
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = BUILD / (LIB.name + ".tmp")
    cmd = [nvcc(), "-shared", "-o", str(tmp)] + [str(o) for o in objs] + [str(blob_o)] + ARCH + ["-lcudart"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    # C++ host drop-in (namespace gpu over the C ABI) and its check program
    host = HERE / "host"
    subprocess.run(["g++", "-std=c++23", "-O2", "-fPIC", "-shared", "-I", str(ROOT / "include"),
                    str(host / "mcl_gpu.cpp"), "-L", str(BUILD), "-lthoth_gpu", "-Wl,-rpath,$ORIGIN",
                    "-o", str(BUILD / "libthoth_mcl_gpu.so")], check=True)
    subprocess.run(["g++", "-std=c++23", "-O2", "-I", str(ROOT / "include"), "-I", str(host),
                    str(host / "host_check.cpp"), "-L", str(BUILD), "-lthoth_mcl_gpu", "-lthoth_gpu",
                    "-Wl,-rpath,$ORIGIN", "-o", str(BUILD / "host_check")], check=True)
    return LIB


if __name__ == "__main__":
    print(build_sanitized() if "--sanitize" in sys.argv else build(verbose="-v" in sys.argv))
