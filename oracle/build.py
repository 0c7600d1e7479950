"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles oracle/nmf_oracle.c into oracle/_lib/liborc.so.
  It is built with ``-ffp-contract=off`` so that no multiply-add is fused on
  either architecture (gcc fuses by default on aarch64); the float
  transcription then gives the same bits on x86-64 and on Arm.
* ``build_ref()`` compiles the reference's own CPU NMF
  (src/examples/FacesNMF/HostNMF.h) from the reference tree, when that tree is
  present, into oracle/_ref/libhostnmf_ref.so.  The only generated source is a
  copy of src/examples/FacesNMF/Matrix.h whose lines 59-80 get their three
  member references qualified with ``this->`` / ``(*this)`` (the file was
  written for MSVC and fails g++'s two-phase lookup) and whose include of
  HostMatrix.h is made absolute.  Everything lands in the git-ignored
  oracle/_ref/.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_lib")
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("GPUNMF_REFERENCE_ROOT", "/root/reference")

CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread"]


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force=False):
    os.makedirs(LIB_DIR, exist_ok=True)
    src = os.path.join(HERE, "nmf_oracle.c")
    out = os.path.join(LIB_DIR, "liborc.so")
    if not force and _newer(out, [src, __file__]):
        return out
    cmd = ["gcc", *CFLAGS, src, "-o", out, "-lm"]
    subprocess.run(cmd, check=True)
    return out


def _patched_matrix_h(src_text, hostmatrix_path):
    lines = src_text.splitlines(keepends=True)
    out = []
    for no, line in enumerate(lines, start=1):
        if 59 <= no <= 80:
            line = re.sub(r"(?<![.>\w])rows\b", "this->rows", line)
            line = re.sub(r"(?<![.>\w])columns\b", "this->columns", line)
            line = line.replace("operator ()(", "(*this)(")
        if '#include "../../memory/HostMatrix.h"' in line:
            line = '#include "%s"\n' % hostmatrix_path
        out.append(line)
    return "".join(out)


def reference_available():
    return os.path.isfile(os.path.join(REFERENCE_ROOT, "src/examples/FacesNMF/HostNMF.h"))


def build_ref(force=False):
    """Build oracle/_ref/libhostnmf_ref.so; returns its path or None."""
    if not reference_available():
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    faces = os.path.join(REFERENCE_ROOT, "src/examples/FacesNMF")
    matrix_src = os.path.join(faces, "Matrix.h")
    shim = os.path.join(HERE, "ref_shim.cpp")
    out = os.path.join(REF_DIR, "libhostnmf_ref.so")
    if not force and _newer(out, [shim, __file__]):
        return out
    with open(matrix_src, "r", encoding="latin-1") as f:
        text = f.read()
    patched = _patched_matrix_h(text, os.path.join(REFERENCE_ROOT, "src/memory/HostMatrix.h"))
    with open(os.path.join(REF_DIR, "Matrix.h"), "w", encoding="latin-1") as f:
        f.write(patched)
    cuda_inc = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"
    cmd = ["g++", "-std=c++14", *CFLAGS, "-w",
           "-I", REF_DIR,                                        # generated Matrix.h first
           "-I", os.path.join(REFERENCE_ROOT, "src/cuda"),       # definitions.h
           "-I", faces,                                          # HostNMF.h
           "-I", cuda_inc,
           shim, "-o", out,
           # HostMemoryManager.h references cudaMemcpy (device copies); the CPU path never calls it
           "-L", os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/lib64", "-lcudart"]
    subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
