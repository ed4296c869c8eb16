"""Measured arithmetic and copy rates of the GPU (roofline ceilings).

    python -m weldform_gb300.probe_rates

Compiles ``csrc/probe_rates.cu`` for sm_103a into ``_build/probe_rates`` (once)
and runs it: FP64 FMA, FP32 FMA, FP64 divide, FP64 square root and FP64->FP32
conversion rates in Gop/s, and a 4 GiB device-to-device copy in GB/s.  The
plain FP64 form's gathers are bound by the FP64 rate, the mixed form's by
memory latency and the copy rate.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "probe_rates.cu")
EXE = os.path.join(HERE, "_build", "probe_rates")


def build() -> str:
    if not os.path.exists(EXE) or os.path.getmtime(EXE) < os.path.getmtime(SRC):
        os.makedirs(os.path.dirname(EXE), exist_ok=True)
        nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", EXE, SRC], check=True)
    return EXE


def main():
    r = subprocess.run([build()], capture_output=True, text=True)
    sys.stdout.write(r.stdout)
    sys.stderr.write(r.stderr)
    sys.exit(r.returncode)


if __name__ == "__main__":
    main()
