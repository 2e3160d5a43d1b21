"""Build recipes for the oracle (test infrastructure only).

* build_oracle(): compiles the CPU restatement oracle/nnet_oracle.cpp into
  oracle/liboracle.so (g++ -O3 -fopenmp -ffp-contract=off).  Runs anywhere.
* build_ref(): compiles the reference's own burn-path sources, as they lie under the
  reference tree, together with oracle/ref_driver.cpp into oracle/_ref/libnnet_ref.so.
  Only possible where the reference tree exists; the reference's CMake is bypassed
  (it requires MPI).  The Helmholtz table is #included by helmholtz.cpp at compile time
  (helmholtz.cpp:92-94), so a one-token stub is compiled in and the stand-in table is
  copied into the reference's arrays at run time by ref_load_helmholtz().

Both use -ffp-contract=off so that no multiply-add is fused on either machine (x86 or
aarch64), keeping the two builds bit-comparable.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
DATA = os.path.join(REPO, "sph-exa-nnet_gb300", "data")
FLAGS = ["-O3", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", "-w"]
# the compiler line of the timed CPU baseline, as reported by bench.py
CPU_FLAGS = "g++ " + " ".join(f for f in FLAGS if f not in ("-fPIC", "-shared", "-w"))


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "nnet_oracle.cpp")
    out = os.path.join(HERE, "liboracle.so")
    deps = [src, os.path.join(DATA, "nnet_network_tables.h")]
    if not force and _newer(out, deps):
        return out
    cmd = ["g++", "-std=c++17", *FLAGS, f"-I{DATA}", src, "-o", out + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def reference_root():
    """The reference tree: $NNET_REFERENCE_ROOT, else the `reference_path` that the benchmark spec at
    the repository root names, else None."""
    root = os.environ.get("NNET_REFERENCE_ROOT")
    if root:
        return root
    try:
        import json
        with open(os.path.join(REPO, "BASELINE.json")) as f:
            return json.load(f).get("reference_path")
    except (OSError, ValueError):
        return None


def build_ref(ref_root=None, force=False):
    ref_root = ref_root or reference_root()
    if not ref_root:
        return None
    inc = os.path.join(ref_root, "include")
    if not os.path.isdir(inc):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libnnet_ref.so")
    par = os.path.join(inc, "nnet", "parameterization")
    srcs = [os.path.join(HERE, "ref_driver.cpp"),
            os.path.join(par, "net14", "net14.cpp"),
            os.path.join(par, "net86", "net86.cpp"),
            os.path.join(par, "net87", "net87.cpp"),
            os.path.join(par, "eos", "helmholtz.cpp")]
    if not force and _newer(out, srcs):
        return out
    stub = os.path.join(outdir, "helm_stub.dat")
    with open(stub, "w") as f:
        f.write("STR(0)\n")
    electron = os.path.join(par, "net87", "electron_rate.dat")
    cmd = ["g++", "-std=c++20", *FLAGS, f"-I{inc}", f"-I{os.path.join(inc, 'nnet', 'parallel')}",
           f'-DHELM_TABLE_PATH="{stub}"', f'-DELECTRON_TABLE_PATH="{electron}"', *srcs, "-o", out + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
