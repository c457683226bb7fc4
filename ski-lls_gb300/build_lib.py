"""Builds libskills_gb300.so (sm_103a) from csrc/ with nvcc, one process per
translation unit in parallel, then links.  Used by __graft_entry__.build()."""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(OUT_DIR, "libskills_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo",
          "-I" + CSRC, "-I" + os.path.join(HERE, "..", "include")]


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(OUT_DIR, "obj", src + ".o")
    cmd = [NVCC, *ARCH, *COMMON, "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cu"):
        cmd += ["--expt-relaxed-constexpr"]
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = [NVCC, *COMMON, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r.returncode, r.stdout + r.stderr


def build(verbose=False, jobs=None):
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)
    srcs = sources()
    objs, errors = [], []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        for src, obj, rc, log in ex.map(lambda s: _compile(s, verbose), srcs):
            if rc != 0:
                errors.append(f"--- {src} ---\n{log}")
            elif verbose and log.strip():
                print(f"--- {src} ---\n{log}")
            objs.append(obj)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


CLI_DIR = os.path.join(HERE, "cli")
CLI_TOOLS = ("ls_qr", "ls_blendenpik_hashing", "ls_blendenpik")


def build_cli():
    """Command-line drivers (cli/*.cpp) over the C++ drop-in header, linked
    against the library; binaries next to it in lib/."""
    inc = os.path.join(os.path.dirname(HERE), "include")
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(NVCC)), "include")
    out = []
    for tool in CLI_TOOLS:
        exe = os.path.join(OUT_DIR, tool)
        cmd = ["g++", "-std=c++17", "-O2", "-I", inc, "-I", CLI_DIR, "-I", cuda_inc,
               os.path.join(CLI_DIR, tool + ".cpp"), "-o", exe, "-L", OUT_DIR, "-lskills_gb300",
               "-Wl,-rpath," + OUT_DIR]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for {tool}:\n" + r.stdout + r.stderr)
        out.append(exe)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    print(build_cli())
