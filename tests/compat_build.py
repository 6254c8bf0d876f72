"""Builds programs against the package-facing compatibility layer (parthenon_gb300/compat)
with nvcc for sm_103a: the layer's headers, the C-ABI header and the library. Test
infrastructure (the layer itself is header-only)."""
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
COMPAT = os.path.join(ROOT, "parthenon_gb300", "compat")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "parthenon_gb300", "_build")
OUT = os.path.join(ROOT, "tests", "cxx", "_build")


def nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def compile_objects(sources, tag, extra=(), include=()):
    """Compile sources in parallel; returns the object paths."""
    os.makedirs(OUT, exist_ok=True)
    procs, objs = [], []
    for src in sources:
        obj = os.path.join(OUT, "%s_%s.o" % (tag, os.path.splitext(os.path.basename(src))[0]))
        cmd = [nvcc(), "-std=c++17", "--extended-lambda", "--expt-relaxed-constexpr", "-x", "cu", "-gencode",
               "arch=compute_103a,code=sm_103a", "-I", COMPAT, "-I", INCLUDE] + \
              [a for d in include for a in ("-I", d)] + list(extra) + ["-c", src, "-o", obj]
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True), cmd))
        objs.append(obj)
    for p, cmd in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), out[-6000:]))
    return objs


def link(objs, name):
    exe = os.path.join(OUT, name)
    cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe] + objs + \
          ["-L", LIBDIR, "-lparthenon_gb300", "-Xlinker", "-rpath", "-Xlinker", LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    return exe
