"""Builds libppgpu.so (CUDA kernels for sm_103a + the C host library) and the ppgpu command-line driver.

Everything is compiled in-tree: objects under patchyparticles_gb300/_build/, the shared library at
patchyparticles_gb300/libppgpu.so, the driver at patchyparticles_gb300/ppgpu. No cmake, one -gencode,
translation units compiled in parallel.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "libppgpu.so")
CLI = os.path.join(HERE, "ppgpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _run_all(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
            raise RuntimeError("build step failed: " + " ".join(c))


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(force=False, verbose=False):
    """Builds the library. PPGPU_DEFINES (e.g. "-DPSTEP=8 -DPPI_TILE_MIN_BLOCKS=4") adds preprocessor
    definitions to the CUDA compile, for tuning measurements; it forces a rebuild."""
    os.makedirs(BUILD, exist_ok=True)
    defines = os.environ.get("PPGPU_DEFINES", "").split()
    force = force or bool(defines)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = "nvcc"
    inc = ["-I", INCLUDE, "-I", CSRC, "-I", os.path.join(cuda, "include")]
    headers = [os.path.join(CSRC, "ppgpu_internal.h"), os.path.join(CSRC, "ppgpu_umma.cuh"), os.path.join(INCLUDE, "ppgpu.h")]
    units = []
    cu_srcs = ["ppgpu_kernels.cu", "ppgpu_mlp.cu"]
    c_srcs = ["ppgpu_host.c"]
    cmds = []
    objs = []
    for s in cu_srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            cmds.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--ptxas-options=-v" if verbose else "-w"] + defines + inc + ["-c", src, "-o", obj])
    for s in c_srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            # -ffp-contract=off: the .rrr reader and the generator must round exactly like the reference
            cmds.append(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=gnu99", "-fPIC", "-Wall", "-Wno-unused-result"] + inc + ["-c", src, "-o", obj])
    cli_src = os.path.join(CSRC, "ppgpu_cli.c")
    cli_obj = os.path.join(BUILD, "ppgpu_cli.c.o")
    have_cli = os.path.exists(cli_src)
    if have_cli and (force or _newer(cli_obj, [cli_src] + headers)):
        cmds.append(["gcc", "-O2", "-ffp-contract=off", "-std=gnu99", "-Wall", "-Wno-unused-result"] + inc + ["-c", cli_src, "-o", cli_obj])
    _run_all(cmds)
    if force or _newer(LIB, objs):
        _run_all([[nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]])
    if have_cli and (force or _newer(CLI, [cli_obj, LIB])):
        _run_all([["gcc", "-o", CLI, cli_obj, "-L", HERE, "-Wl,-rpath,$ORIGIN", "-lppgpu", "-lm"]])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
