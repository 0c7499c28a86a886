"""Build recipe of the native library (libpxdock_gb300.so), in-tree.

nvcc compiles every csrc/*.cu (and the host-only csrc/*.cpp) for sm_103a in parallel and
links one shared library
with the C ABI of include/pxdock_gb300.h. A content hash of sources and flags makes a
rebuild a no-op when nothing changed.
"""
import concurrent.futures
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
CSRC = os.path.join(PKG_ROOT, "csrc")
REPO = os.path.dirname(PKG_ROOT)
OUT_DIR = os.path.join(HERE, "_native")
LIB_NAME = "libpxdock_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code without fused multiply-add contraction, so that its FP64 results (the pose
# clustering rule, conversions) are the same on x86-64 and aarch64 hosts
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr",
              "-Xptxas", "-v"] + ARCH


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _digest(files, flags):
    h = hashlib.sha256()
    extra = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    extra += [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]
    for path in sorted(files + extra):
        h.update(path.encode())
        with open(path, "rb") as f:
            h.update(f.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def lib_path():
    return os.path.join(OUT_DIR, LIB_NAME)


def build(verbose=False, jobs=None):
    """Compiles and links the library unless an up-to-date copy exists; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    files = sources()
    digest = _digest(files, NVCC_FLAGS)
    stamp = os.path.join(OUT_DIR, "build.stamp")
    out = lib_path()
    if os.path.exists(out) and os.path.exists(stamp) and open(stamp).read() == digest:
        return out
    cc = nvcc()
    objs = []
    logs = {}

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")
        cmd = [cc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        return src, obj, r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs or len(files)) as ex:
        for src, obj, log in ex.map(compile_one, files):
            objs.append(obj)
            logs[os.path.basename(src)] = log
    with open(os.path.join(OUT_DIR, "ptxas.log"), "w") as f:
        for name in sorted(logs):
            f.write("== %s\n%s\n" % (name, logs[name]))
    tmp = out + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, out)
    with open(stamp, "w") as f:
        f.write(digest)
    if verbose:
        print(open(os.path.join(OUT_DIR, "ptxas.log")).read())
    return out


if __name__ == "__main__":
    print(build(verbose=True))
