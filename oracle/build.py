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
* ``build_ref_faces()`` compiles the reference's own FacesNMF image loader:
  the definitions of ``CFacesNMFDlg::FolderHasImages`` and
  ``CFacesNMFDlg::LoadImage`` are copied unchanged out of
  src/examples/FacesNMF/FacesNMFDlg.cpp into oracle/_ref/faces_dlg_methods.inc
  and built with oracle/ref_faces_shim.cpp (plain C++ stand-ins for the MFC
  names they use) into oracle/_ref/libfaces_ref.so.
* ``stage_ref_gpu_sources()`` copies the reference's sources for its GPU NMF
  classes (the files in REF_GPU_FILES, unchanged, keeping their relative
  paths) into oracle/_ref/gpu_src/, and ``build_ref_gpu()`` compiles them with
  oracle/ref_gpu_shim.cu for sm_103a against cuBLAS into
  oracle/_ref/libref_gpu_nmf.so.  The copies exist because the machine with
  the GPU has no reference tree: the recipe runs there from the staged copy.
  They are git-ignored build inputs, never part of the repository.
* ``stage_faces_images()`` copies the data set (src/examples/FacesNMF/images,
  2429 P5 files of 19 x 19) into oracle/_ref/faces_images/, where the GPU
  tests find it on a machine without the reference tree.

The reference root is one setting: the environment variable
GPUNMF_REFERENCE_ROOT, else DEFAULT_REFERENCE_ROOT below.  Without a reference
tree there, every builder here returns None and the tests that need the
reference's own code skip; the committed golden vectors carry the checks.
"""
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_lib")
REF_DIR = os.path.join(HERE, "_ref")
DEFAULT_REFERENCE_ROOT = "/root/reference"
REFERENCE_ROOT = os.environ.get("GPUNMF_REFERENCE_ROOT", DEFAULT_REFERENCE_ROOT)
FACES_IMAGES = os.path.join(REF_DIR, "faces_images")

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


def _definition(text, signature):
    """The text of the function definition that starts with `signature`, through its closing brace."""
    start = text.index(signature)
    open_at = text.index("{", start)
    depth = 0
    for i in range(open_at, len(text)):
        if text[i] == "{":
            depth += 1
        elif text[i] == "}":
            depth -= 1
            if depth == 0:
                return text[start:i + 1]
    raise ValueError("unbalanced braces after " + signature)


def build_ref_faces(force=False):
    """Build oracle/_ref/libfaces_ref.so from the reference's loader; returns its path or None."""
    if not reference_available():
        return None
    build_ref(force)   # writes the generated Matrix.h the loader's Matrix<cudafloat> needs
    faces = os.path.join(REFERENCE_ROOT, "src/examples/FacesNMF")
    shim = os.path.join(HERE, "ref_faces_shim.cpp")
    out = os.path.join(REF_DIR, "libfaces_ref.so")
    if not force and _newer(out, [shim, __file__]):
        return out
    with open(os.path.join(faces, "FacesNMFDlg.cpp"), "r", encoding="latin-1") as f:
        text = f.read()
    methods = [_definition(text, "bool CFacesNMFDlg::FolderHasImages("),
               _definition(text, "bool CFacesNMFDlg::LoadImage(")]
    with open(os.path.join(REF_DIR, "faces_dlg_methods.inc"), "w", encoding="latin-1") as f:
        f.write("// copied unchanged from src/examples/FacesNMF/FacesNMFDlg.cpp by oracle/build.py\n")
        f.write("\n\n".join(methods) + "\n")
    cmd = ["g++", "-std=c++14", *CFLAGS, "-w",
           "-I", REF_DIR,
           "-I", os.path.join(REFERENCE_ROOT, "src/cuda"),
           "-I", os.path.join(REFERENCE_ROOT, "src/memory"),
           "-I", os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include",
           shim, "-o", out,
           "-L", os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/lib64", "-lcudart"]
    subprocess.run(cmd, check=True)
    return out


REF_GPU_DIR = os.path.join(REF_DIR, "gpu_src")
REF_GPU_FILES = [
    "src/algorithms/nmf/nmf_base.h",
    "src/algorithms/nmf/nmf_multiplicative_euclidian.h",
    "src/algorithms/nmf/nmf_multiplicative_euclidian.cpp",
    "src/algorithms/nmf/nmf_multiplicative_divergence.h",
    "src/algorithms/nmf/nmf_multiplicative_divergence.cpp",
    "src/cuda/definitions.h",
    "src/cuda/nmf/nmf_kernels.h",
    "src/cuda/nmf/nmf_kernels.cu",
    "src/cuda/nmf/nmf_kernels_quality.cu",
    "src/common/CudaStreams.h",
    "src/common/Utilities.h",
    "src/common/config.h",
] + ["src/memory/" + h for h in ("BaseArray.h", "BaseMatrix.h", "DeviceAccessibleVariable.h", "DeviceArray.h",
                                 "DeviceMatrix.h", "DeviceMemoryManager.h", "HostArray.h", "HostMatrix.h",
                                 "HostMemoryManager.h", "MemoryManager.h")]
# the definitions the reference's CMakeLists.txt:119-124 sets for compute capability >= 3.0
REF_GPU_DEFINES = ["-DCUDA_MAX_THREADS_PER_BLOCK=1024", "-DCUDA_MAX_GRID_X_DIM=2147483647"]


def stage_ref_gpu_sources():
    """Copy REF_GPU_FILES into oracle/_ref/gpu_src/; returns that folder, or None without sources."""
    if os.path.isdir(os.path.join(REFERENCE_ROOT, "src")):
        for rel in REF_GPU_FILES:
            src, dst = os.path.join(REFERENCE_ROOT, rel), os.path.join(REF_GPU_DIR, rel)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            if not (os.path.isfile(dst) and open(src, "rb").read() == open(dst, "rb").read()):
                shutil.copyfile(src, dst)
    if all(os.path.isfile(os.path.join(REF_GPU_DIR, rel)) for rel in REF_GPU_FILES):
        return REF_GPU_DIR
    return None


def build_ref_gpu(force=False):
    """Build oracle/_ref/libref_gpu_nmf.so from the staged sources; returns its path or None."""
    root = stage_ref_gpu_sources()
    if root is None:
        return None
    shim = os.path.join(HERE, "ref_gpu_shim.cu")
    out = os.path.join(REF_DIR, "libref_gpu_nmf.so")
    srcs = [os.path.join(root, rel) for rel in REF_GPU_FILES if rel.endswith((".cpp", ".cu"))]
    if not force and _newer(out, [shim, __file__] + srcs):
        return out
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
           "-Xcompiler", "-fPIC", "-w", *REF_GPU_DEFINES, "-I", os.path.join(root, "src"),
           shim, *srcs, "-o", out, "-lcublas"]
    subprocess.run(cmd, check=True)
    return out


def stage_faces_images():
    """Copy the FacesNMF data set into oracle/_ref/faces_images/; returns the folder or None."""
    src = os.path.join(REFERENCE_ROOT, "src/examples/FacesNMF/images")
    if not os.path.isdir(src):
        return FACES_IMAGES if os.path.isdir(FACES_IMAGES) else None
    os.makedirs(FACES_IMAGES, exist_ok=True)
    for name in sorted(os.listdir(src)):
        if not name.endswith(".pgm"):
            continue
        dst = os.path.join(FACES_IMAGES, name)
        if not os.path.exists(dst):
            shutil.copyfile(os.path.join(src, name), dst)
    return FACES_IMAGES


def backslash_folder(folder, workdir):
    """A folder name F such that F + "\\" + "faceNNNNN.pgm" names each image of `folder`.

    The reference loader joins folder and file with a backslash
    (FacesNMFDlg.cpp:315,334,417); on Linux that is part of one file name, so
    `workdir` receives links named 'x\\faceNNNNN.pgm' to the images."""
    os.makedirs(workdir, exist_ok=True)
    for name in os.listdir(folder):
        if name.startswith("face") and name.endswith(".pgm"):
            link = os.path.join(workdir, "x\\" + name)
            if not os.path.lexists(link):
                os.symlink(os.path.abspath(os.path.join(folder, name)), link)
    return os.path.join(workdir, "x")


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_ref_faces(force="--force" in sys.argv))
    print(stage_faces_images())
    print(build_ref_gpu(force="--force" in sys.argv))
