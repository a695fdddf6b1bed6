"""Build and run peak_probe.cu (FP64/FP32 arithmetic and copy peaks).

    python -m dplr_gb300.diag.peak_probe
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main() -> int:
    out_dir = os.path.join(os.path.dirname(HERE), "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "peak_probe")
    subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                           os.path.join(HERE, "peak_probe.cu")])
    return subprocess.call([exe])


if __name__ == "__main__":
    sys.exit(main())
