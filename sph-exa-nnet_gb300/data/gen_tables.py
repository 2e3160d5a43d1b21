"""Regenerate nnet_network_tables.h from the reference's network definition headers.

Compiles dump_reference_tables.cpp against the reference include tree (which is only
present on the development machine) and writes its output beside this script.  The
generated header is committed; the build never needs the reference at run time.

usage: python gen_tables.py [REFERENCE_ROOT]
(default: $NNET_REFERENCE_ROOT, else the reference_path that the benchmark spec at the repository
root names)
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root():
    root = os.environ.get("NNET_REFERENCE_ROOT")
    if root:
        return root
    with open(os.path.join(HERE, "..", "..", "BASELINE.json")) as f:
        return json.load(f)["reference_path"]


def main(ref_root=None):
    ref_root = ref_root or reference_root()
    inc = os.path.join(ref_root, "include")
    par = os.path.join(inc, "nnet", "parameterization")
    electron = os.path.join(par, "net87", "electron_rate.dat")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "dump")
        cmd = ["g++", "-O1", "-std=c++20", "-w", f"-I{inc}",
               f'-DELECTRON_TABLE_PATH="{electron}"',
               os.path.join(HERE, "dump_reference_tables.cpp"),
               os.path.join(par, "net14", "net14.cpp"),
               os.path.join(par, "net86", "net86.cpp"),
               os.path.join(par, "net87", "net87.cpp"),
               "-o", exe]
        subprocess.run(cmd, check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    path = os.path.join(HERE, "nnet_network_tables.h")
    with open(path, "w") as f:
        f.write(out)
    print(f"wrote {path} ({len(out)} bytes)")


if __name__ == "__main__":
    main(*sys.argv[1:])
