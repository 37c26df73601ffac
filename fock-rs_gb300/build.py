"""Build the GB300 library in-tree: generate the class kernels, compile every
translation unit with nvcc for sm_103a in parallel, link one shared library.

Output: fock-rs_gb300/lib/libfock_gb300.so  (C ABI of include/fock_gb300.h)
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
GEN = os.path.join(CSRC, "gen")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libfock_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LMAX = int(os.environ.get("FOCK_GB300_LMAX", "2"))


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _sources():
    srcs = [os.path.join(CSRC, f) for f in ("fock_api.cu", "md_device.cu", "scf_device.cu", "noalloc.cu", "eigen.cu",
                                            "loaders.cpp")]
    srcs += sorted(os.path.join(GEN, f) for f in os.listdir(GEN) if f.startswith("inst_") and f.endswith(".cu"))
    return srcs


def _includes(path, seen):
    """Quoted #include files of path, transitively (the files a translation unit depends on)."""
    if path in seen or not os.path.isfile(path):
        return
    seen.add(path)
    with open(path, errors="replace") as f:
        for line in f:
            t = line.strip()
            if t.startswith("#include") and '"' in t:
                name = t.split('"')[1]
                _includes(os.path.normpath(os.path.join(os.path.dirname(path), name)), seen)


def _deps_mtime(src):
    seen = set()
    _includes(src, seen)
    return max(os.path.getmtime(p) for p in seen)


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", CSRC, "--expt-relaxed-constexpr"] + \
        os.environ.get("FOCK_GB300_NVCC_FLAGS", "").split()


def _compile(src, verbose):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if not verbose and os.path.exists(obj) and os.path.getmtime(obj) >= _deps_mtime(src):
        return obj
    cmd = [nvcc()] + _flags() + ["-c", src, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def write_ref_lut():
    """gen/ref_lut.inc: the reference's stored Boys table (data/boys_ref_lut.json)
    as a C array for the reference-compatible mode."""
    import json
    with open(os.path.join(HERE, "data", "boys_ref_lut.json")) as f:
        vals = json.load(f)["values"]
    assert len(vals) == 200
    body = ",\n".join("  %r" % float(v) for v in vals)
    text = ("// Generated by build.py from data/boys_ref_lut.json. Do not edit.\n"
            "static const double kRefBoysLut[200] = {\n%s};\n" % body)
    path = os.path.join(GEN, "ref_lut.inc")
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)


def build(verbose=False, jobs=None):
    sys.path.insert(0, CSRC)
    import gen_eri  # noqa
    sys.path.pop(0)
    os.makedirs(GEN, exist_ok=True)
    # generate into a scratch folder and copy only the files that changed, so
    # that unchanged translation units keep their objects
    tmp = GEN + ".tmp"
    shutil.rmtree(tmp, ignore_errors=True)
    gen_eri.main(tmp, LMAX)
    fresh = set(os.listdir(tmp))
    for f in os.listdir(GEN):
        if f.startswith(("inst_", "cls_")) and f not in fresh:
            os.remove(os.path.join(GEN, f))
    for f in fresh:
        new, old = os.path.join(tmp, f), os.path.join(GEN, f)
        with open(new) as a:
            text = a.read()
        if not os.path.exists(old) or open(old).read() != text:
            shutil.copyfile(new, old)
    shutil.rmtree(tmp, ignore_errors=True)
    write_ref_lut()
    os.makedirs(OBJ, exist_ok=True)
    # objects built with other flags are stale
    stamp = os.path.join(OBJ, "flags.txt")
    flags = " ".join(_flags())
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        for f in os.listdir(OBJ):
            if f.endswith(".o"):
                os.remove(os.path.join(OBJ, f))
        with open(stamp, "w") as f:
            f.write(flags)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + [
        "-L", cuda_lib, "-lcublas", "-lcusolver", "-Xlinker", "-rpath=" + cuda_lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
