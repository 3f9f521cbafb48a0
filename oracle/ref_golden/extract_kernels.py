"""Build step of `make -C oracle ref`: collect the reference's kernel functions.

Copies fixed line ranges of the reference's CUDA sources -- the kernels and
__device__ helpers of the LC2 path, nothing of the host classes -- into
oracle/_ref/ref_kernels.inc (git-ignored), where kernel_emu.cpp compiles them
as host C++ under a CUDA-semantics emulator. Each range is checked against
the line it must start with, so a different reference revision fails loudly
instead of compiling the wrong code.

    python extract_kernels.py <reference root> <output .inc>
"""
import sys

RANGES = [
    # (file, first line, last line, expected start of the first line)
    ("src/Interpolator/interpolator.cuh", 27, 41, "//3D:"),
    ("src/Interpolator/interpolator.cu", 69, 232, "__global__ void Interpolate_3Dkernel("),
    ("src/cu_LC2/cu_lc2_2d.cu", 25, 480, "__global__ void gradient2DSobelKernel("),
    ("src/cu_LC2/cu_lc2_3d.cu", 100, 618, "__global__ void gradient3DSobelKernel("),
    ("src/cu_LC2/cu_lc2_3d.cu", 625, 827, "__device__ float conjugateGradient_3Dkernel_ForGlobalMemory("),
]


def main(ref_root: str, out_path: str) -> None:
    parts = []
    for rel, a, b, head in RANGES:
        with open(f"{ref_root}/{rel}") as f:
            lines = f.read().splitlines()
        first = lines[a - 1].strip()
        if not first.startswith(head):
            sys.exit(f"{rel}:{a}: expected '{head}', found '{first}'")
        parts.append(f"// ---- {rel}:{a}-{b}\n#line {a} \"{rel}\"\n")
        parts.append("\n".join(lines[a - 1:b]) + "\n")
    with open(out_path, "w") as f:
        f.write("".join(parts))


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
