"""Build libpypde_gb300.so in place with nvcc for sm_103a.

Every translation unit of pypde_gb300/csrc is compiled in parallel, then
linked into one shared library with the CUDA runtime linked statically, so
that the library loads (and reports errors) on a machine without a GPU
driver.  Kernels are compiled with --fmad=false: the plain FP64 form is
bit-faithful to the host restatement of the reference algorithm, which
fuses a multiply and an add only where both sides call fma() explicitly.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpypde_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
ORDERS = (1, 2, 3)  # orders of the ahead-of-time kernels (MAXN in runtime.h)


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _needs(obj, src_paths):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in src_paths)


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "pypde_gb300.h"))
    flags = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
             "-Xcompiler", "-ffp-contract=off",
             "-Xcompiler", "-fno-strict-aliasing", ARCH, "-Xptxas", "-O3"]
    cmds = []
    objs = []
    for f in sources():
        src = os.path.join(CSRC, f)
        # an instantiation unit is compiled once per order, so that the
        # (system, order) pairs compile in parallel
        variants = ([(f"{f}.n{n}.o", [f"-DPYPDE_ORDER={n}"]) for n in ORDERS]
                    if f.startswith("inst_") else [(f + ".o", [])])
        for oname, extra in variants:
            obj = os.path.join(OBJ, oname)
            objs.append(obj)
            if _needs(obj, [src] + headers + [__file__]):
                cmds.append([nv, *flags, *extra, "-x", "cu", "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failed = []
    # the longest units first, so that they do not finish last
    cmds.sort(key=lambda c: ("inst_cattaneo" not in c[-3], "-DPYPDE_ORDER=3" not in c))
    with ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        for cmd, r in ex.map(run, cmds):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                failed.append(cmd[-3])
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(failed))
    if cmds or not os.path.exists(LIB):
        link = [nv, "-shared", ARCH, "-cudart", "static", "-o", LIB, *objs, "-ldl", "-lpthread"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
