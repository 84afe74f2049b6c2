"""Test infrastructure: builds the oracle's CPU port (oracle/_build/lts_port) with g++ + OpenMP.

-ffp-contract=off keeps float expressions unfused on every CPU (aarch64 g++ would otherwise
contract a*b+c into FMA), so the port rounds as the reference's x86 host build does.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(ROOT, "oracle", "_build")


def build():
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "lts_port")
    csrc = os.path.join(ROOT, "lighttransportsimulation_gb300", "csrc")
    srcs = [os.path.join(HERE, "lts_port.cpp"), os.path.join(csrc, "host_scene.cpp"), os.path.join(csrc, "image_io.cpp"),
            os.path.join(csrc, "jpeg_io.cpp")]
    deps = srcs + [os.path.join(HERE, "lts_rng.h"), os.path.join(ROOT, "include", "lts_capi.h"),
                   os.path.join(csrc, "host_scene.hpp"), os.path.join(csrc, "image_io.hpp")]
    if os.path.exists(exe) and all(os.path.getmtime(d) <= os.path.getmtime(exe) for d in deps):
        return exe
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-o", exe + ".tmp", *srcs]
    subprocess.run(cmd, check=True)
    os.replace(exe + ".tmp", exe)
    return exe


if __name__ == "__main__":
    print(build())
    sys.exit(0)
