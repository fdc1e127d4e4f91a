"""In-tree build of the native parts (no cmake, no setuptools).

Products (all git-ignored, rebuilt on each host):
  meep_gb300/lib/libmfd.so            CUDA engine + C ABI (include/mfd.h)
  meep_gb300/lib/libmeep_gb300.so     C++ drop-in (include/meep_gb300/meep.hpp), realnum = double
  meep_gb300/lib/libmeep_gb300_single.so  the same with realnum = float
  meep_gb300/lib/golden_driver{64,32} the golden-fixture driver linked against them
Test infrastructure (built when asked, see build_oracle):
  oracle/_build/liboracle_mfd.so      same C ABI over the CPU oracle backend
  oracle/_ref/...                     reference core (only where its sources exist)
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "meep_gb300")
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "lib")
INC = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "include", "meep_gb300"),
       "-I" + CSRC, "-I" + os.path.join(PKG, "workloads")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# checkout of the reference (its src/ directory is compiled into oracle/_ref
# by oracle/ref/Makefile); unset: the reference core is not built
REFERENCE = os.environ.get("MEEP_REFERENCE", "")


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, cwd=ROOT):
    res = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), res.stdout[-4000:]))
    return res.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(ROOT, "include", "mfd.h"), os.path.join(ROOT, "include", "meep_gb300", "meep.hpp"),
              os.path.join(ROOT, "include", "meep_gb300", "mgb.h")]
    return files


def build_engine(force=False, verbose=False):
    """Compile the CUDA engine and the C ABI into libmfd.so, and the C++
    drop-in into libmeep_gb300.so / libmeep_gb300_single.so."""
    os.makedirs(LIB, exist_ok=True)
    so = os.path.join(LIB, "libmfd.so")
    deps = _deps()
    if not force and not _newer(so, deps):
        return so
    nvcc = _nvcc()
    objdir = os.path.join(LIB, "obj")
    os.makedirs(objdir, exist_ok=True)
    jobs = []
    cu_common = [nvcc] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC"] + INC
    jobs.append(cu_common + ["--fmad=false", "-c", os.path.join(CSRC, "mfd_cuda_f64.cu"),
                             "-o", os.path.join(objdir, "mfd_cuda_f64.o")])
    jobs.append(cu_common + ["-c", os.path.join(CSRC, "mfd_cuda_f32.cu"),
                             "-o", os.path.join(objdir, "mfd_cuda_f32.o")])
    jobs.append(cu_common + ["-c", os.path.join(CSRC, "mfd_noalloc.cu"),
                             "-o", os.path.join(objdir, "mfd_noalloc.o")])
    jobs.append(cu_common + ["--fmad=false", "-c", os.path.join(CSRC, "mfd_subpixel.cu"),
                             "-o", os.path.join(objdir, "mfd_subpixel.o")])
    jobs.append(cu_common + ["-c", os.path.join(CSRC, "mfd_near2far.cu"),
                             "-o", os.path.join(objdir, "mfd_near2far.o")])
    for src in ("mfd_plan.cpp", "mfd_capi.cpp", "sphere_quadrature.cpp"):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"] + INC +
                    ["-c", os.path.join(CSRC, src), "-o", os.path.join(objdir, src.replace(".cpp", ".o"))])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    objs = [os.path.join(objdir, f) for f in ("mfd_cuda_f64.o", "mfd_cuda_f32.o", "mfd_noalloc.o",
                                               "mfd_subpixel.o", "mfd_near2far.o", "mfd_plan.o", "mfd_capi.o",
                                               "sphere_quadrature.o")]
    _run([nvcc] + ARCH + ["-shared", "-o", so] + objs + ["-lcudart"])
    api = [os.path.join(CSRC, "meep_api.cpp"), os.path.join(CSRC, "meep_pyshim.cpp")]
    links = []
    for name, flag in (("libmeep_gb300.so", []), ("libmeep_gb300_single.so", ["-DMEEP_SINGLE=1"])):
        links.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off"] + flag + INC +
                     ["-o", os.path.join(LIB, name)] + api + ["-L" + LIB, "-lmfd", "-Wl,-rpath," + LIB])
    with ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, links))
    return so


def build_drivers(force=False):
    """Golden-fixture driver compiled against the drop-in header and the engine."""
    so = build_engine()
    src = os.path.join(ROOT, "tests", "golden", "golden_driver.cpp")
    outs = []
    jobs = []
    for bits, flag in ((64, []), (32, ["-DMEEP_SINGLE=1"])):
        exe = os.path.join(LIB, "golden_driver%d" % bits)
        outs.append(exe)
        if not force and not _newer(exe, [src, so] + _deps()):
            continue
        lib = "-lmeep_gb300" if bits == 64 else "-lmeep_gb300_single"
        jobs.append(["g++", "-O2", "-std=c++17", "-ffp-contract=off"] + flag + INC +
                    ["-o", exe, src, "-L" + LIB, lib, "-lmfd", "-Wl,-rpath," + LIB])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    return outs


def build_bench(force=False):
    """Benchmark driver (meep_gb300/workloads/bench_main.cpp) over the engine."""
    so = build_engine()
    src = os.path.join(PKG, "workloads", "bench_main.cpp")
    hdr = os.path.join(PKG, "workloads", "cases.hpp")
    outs, jobs = [], []
    for bits, flag in ((64, []), (32, ["-DMEEP_SINGLE=1"])):
        exe = os.path.join(LIB, "bench_main%d" % bits)
        outs.append(exe)
        if not force and not _newer(exe, [src, hdr, so] + _deps()):
            continue
        lib = "-lmeep_gb300" if bits == 64 else "-lmeep_gb300_single"
        jobs.append(["g++", "-O2", "-std=c++17", "-ffp-contract=off"] + flag + INC +
                    ["-o", exe, src, "-L" + LIB, lib, "-lmfd", "-Wl,-rpath," + LIB])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    return outs


def build_oracle():
    """CPU oracle (test infrastructure)."""
    _run(["make", "-C", os.path.join(ROOT, "oracle"), "-j8"])
    return os.path.join(ROOT, "oracle", "_build", "liboracle_mfd.so")


def build_reference():
    """Reference core, only where its sources are present: MEEP_REFERENCE
    names the reference checkout (test infrastructure, never on the GPU
    host)."""
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "src")):
        return None
    _run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), "-j8", "REF=" + REFERENCE])
    return os.path.join(ROOT, "oracle", "_ref")


if __name__ == "__main__":
    print(build_engine(force="--force" in sys.argv, verbose=True))
