"""Recipe: compile the reference's own CUDA tile-processor kernels into a cubin.

TEST INFRASTRUCTURE ONLY.  The reference GPU kernels (convert_correct_tiles,
imclt_rbg) live in src/main/resources/{dtt8x8.cuh,TileProcessor.cuh} and are
normally compiled by NVRTC at run time with a block of #defines prepended
(GPUTileProcessor.java:262-295).  This recipe does the same with nvcc, for
sm_103a, reading the sources where they lie in the reference checkout
(the directory named by the environment variable TP_REFERENCE_DIR, default
/root/reference) and writing only into oracle/_ref/ (git-ignored).  The cubin is device code only; the GPU
box loads it through the CUDA driver API (oracle/ref_gpu.py) to produce the
golden vectors committed under tests/golden/.  Nothing of the reference source
is copied into the repository.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("TP_REFERENCE_DIR", "/root/reference")
REF_RES = os.path.join(REF_DIR, "src", "main", "resources")


def reference_present():
    return os.path.isdir(REF_RES)
OUT_DIR = os.path.join(HERE, "_ref")

# compile-time geometry of the golden scene (GPUTileProcessor #defines)
GOLDEN_GEOM = dict(IMG_WIDTH=128, IMG_HEIGHT=96)


def cubin_path(width=GOLDEN_GEOM["IMG_WIDTH"], height=GOLDEN_GEOM["IMG_HEIGHT"]):
    return os.path.join(OUT_DIR, "tp_ref_%dx%d.cubin" % (width, height))


def defines(width, height):
    d = dict(JCUDA=1, DTT_SIZE=8, THREADSX=8, NUM_CAMS=4, NUM_COLORS=3, IMG_WIDTH=width, IMG_HEIGHT=height,
             KERNELS_HOR=width // 16 + 2, KERNELS_VERT=height // 16 + 2, KERNELS_LSTEP=4, THREADS_PER_TILE=8,
             TILES_PER_BLOCK=4, IMCLT_THREADS_PER_TILE=16, IMCLT_TILES_PER_BLOCK=4)
    return "".join("#define %s %s\n" % (k, v) for k, v in d.items())


def build(width=GOLDEN_GEOM["IMG_WIDTH"], height=GOLDEN_GEOM["IMG_HEIGHT"], force=False):
    if not reference_present():
        return None  # reference sources only exist on the build machine
    os.makedirs(OUT_DIR, exist_ok=True)
    out = cubin_path(width, height)
    srcs = [os.path.join(REF_RES, f) for f in ("dtt8x8.cuh", "TileProcessor.cuh")]
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(map(os.path.getmtime, srcs + [__file__])):
        return out
    gen = os.path.join(OUT_DIR, "tp_ref_%dx%d.cu" % (width, height))
    with open(gen, "w") as f:
        f.write(defines(width, height))
        f.write('#include "dtt8x8.cuh"\n#include "TileProcessor.cuh"\n')
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w", "-I", REF_RES,
           "-o", out + ".tmp", gen]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
