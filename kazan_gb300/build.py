"""Build the native parts of kazan_gb300 in-tree (kazan_gb300/_build/).

  kz_pipeline.cubin    relocatable sm_103a object with the pipeline kernels (nvcc -rdc -cubin); the
                       driver JIT-links it with each pipeline set's shader PTX at run time
  kz_tex.cubin         relocatable object with the texture sampling functions the shaders call, built
                       within 64 registers per thread (linked with the same PTX)
  libkazan_driver.so   the Vulkan driver (ICD) + shader compiler + PTX backend, C ABI
                       (include/kazan_driver.h, include/kz_shader_backend.h); CUDA runtime linked
                       statically, so the library loads on a machine without a GPU driver; it also
                       carries kz_noalloc.o, the allocation-free entry point (pipeline kernels compiled
                       with a fixed pass-through colour stage)
  libkz_scene.so       seeded synthetic scene generators

Host code is plain C/C++17 with no architecture-specific flags (it builds on x86_64 and aarch64).
"""
import concurrent.futures
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

DRIVER_SOURCES = [
    "icd/kz_icd.cpp",
    "icd/kz_cmd.cpp",
    "shader/kz_spirv.cpp",
    "shader/kz_spirv_to_ir.cpp",
    "shader/kz_ptx_backend.cpp",
    "shader/kz_backend_api.cpp",
]
HEADERS = [
    "kz_raster_abi.h",
    "kz_srgb_table.h",
    "icd/kz_icd.h",
    "shader/kz_ir.h",
    "shader/kz_spirv.h",
    "shader/kz_shader_backend_impl.h",
]


def _newer(out, inputs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(i) > t for i in inputs)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _include_deps():
    inc = os.path.join(ROOT, "include")
    return [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(inc, f) for f in os.listdir(inc)]


def pipeline_object(verbose=False):
    src = os.path.join(CSRC, "raster", "kz_pipeline.cu")
    out = os.path.join(OUT, "kz_pipeline.cubin")
    if _newer(out, [src, os.path.join(CSRC, "kz_raster_abi.h"), os.path.join(CSRC, "kz_srgb_table.h")]):
        cmd = [NVCC, "-rdc=true", "-cubin"] + ARCH + ["-O3", "-lineinfo", "-fmad=false", "-o", out, src]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        log = _run(cmd)
        if verbose:
            sys.stdout.write(log)
    return out


def texture_object(verbose=False):
    """kz_tex.cubin: the texture sampling functions the shaders call, within 64 registers per thread"""
    src = os.path.join(CSRC, "raster", "kz_tex.cu")
    out = os.path.join(OUT, "kz_tex.cubin")
    if _newer(out, [src, os.path.join(CSRC, "kz_raster_abi.h"), os.path.join(CSRC, "kz_srgb_table.h")]):
        cmd = [NVCC, "-rdc=true", "-cubin"] + ARCH + ["-O3", "-lineinfo", "-fmad=false", "-maxrregcount=64", "-o", out,
                                                     src]
        log = _run(cmd)
        if verbose:
            sys.stdout.write(log)
    return out


def _compile_cpp(src):
    obj = os.path.join(OUT, "obj", os.path.basename(src).replace(".cpp", ".o"))
    if _newer(obj, [src] + _include_deps()):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", os.path.join(CUDA, "include"),
              "-c", src, "-o", obj])
    return obj


def _compile_noalloc():
    src = os.path.join(CSRC, "raster", "kz_noalloc.cu")
    obj = os.path.join(OUT, "obj", "kz_noalloc.o")
    deps = [src, os.path.join(CSRC, "raster", "kz_pipeline.cu"), os.path.join(CSRC, "raster", "kz_exact.h"),
            os.path.join(CSRC, "kz_raster_abi.h"), os.path.join(ROOT, "include", "kazan_driver.h")]
    if _newer(obj, deps):
        _run([NVCC, "-c", "-std=c++17"] + ARCH + ["-O3", "-lineinfo", "-fmad=false", "-I", os.path.join(ROOT, "include"),
             "-Xcompiler", "-fPIC,-fvisibility=hidden", "-o", obj, src])
    return obj


def driver_library():
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in DRIVER_SOURCES]
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs) + 1) as ex:
        noalloc = ex.submit(_compile_noalloc)
        objs = list(ex.map(_compile_cpp, srcs)) + [noalloc.result()]
    out = os.path.join(OUT, "libkazan_driver.so")
    if _newer(out, objs):
        lib = os.path.join(CUDA, "lib64")
        _run(["g++", "-shared", "-o", out] + objs +
             [os.path.join(lib, "libcudart_static.a"), "-L" + lib, "-lnvJitLink", "-ldl", "-lpthread", "-lrt",
              "-Wl,-rpath," + lib, "-Wl,--no-undefined"])
    return out


def scene_library():
    src = os.path.join(CSRC, "scene", "kz_scene.c")
    out = os.path.join(OUT, "libkz_scene.so")
    if _newer(out, [src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-fvisibility=hidden", "-o", out, src, "-lm"])
    return out


def build_all(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(pipeline_object, verbose), ex.submit(texture_object, verbose), ex.submit(driver_library),
                ex.submit(scene_library)]
        return [f.result() for f in futs]


if __name__ == "__main__":
    for p in build_all(verbose="-v" in sys.argv):
        print(p)
