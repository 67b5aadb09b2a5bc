"""Builds the C oracle (test infrastructure) into oracle/_build/.

Two builds of the same source:
  libpsf_oracle.so       -O2 -ffp-contract=off : the parity checker (bit-exact
                         with the reference's operation order on any host)
  libpsf_oracle_fast.so  -O3 -fopenmp          : the CPU baseline, the
                         reference's own stock flags (README: g++ -O3 -fopenmp)
and the network oracle of the learned preconditioner:
  libunet_oracle.so      -O2                   : U-Net forward/backward checker
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# where the PANSFEM2 source tree lies, if anywhere (the reference harness and the golden
# fixtures are built from it; nothing at run time needs it)
REFERENCE_ROOT = os.environ.get("PANSFEM2_REF", "/root/reference")
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "psf_oracle.c")
USRC = os.path.join(HERE, "unet_oracle.c")


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    jobs = [
        [cc, "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c11",
         SRC, "-o", os.path.join(OUT, "libpsf_oracle.so"), "-lm"],
        [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11",
         SRC, "-o", os.path.join(OUT, "libpsf_oracle_fast.so"), "-lm"],
        [cc, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
         USRC, "-o", os.path.join(OUT, "libunet_oracle.so"), "-lm"],
    ]
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode())
            raise RuntimeError("oracle build failed: " + " ".join(j))
        if verbose and out:
            sys.stderr.write(out.decode())
    return OUT


def reference_present(ref_root=None):
    return os.path.isdir(os.path.join(ref_root or REFERENCE_ROOT, "src"))


def build_reference(ref_root=None):
    """Builds oracle/_ref/ from the reference sources when they are present."""
    ref_root = ref_root or REFERENCE_ROOT
    if not reference_present(ref_root):
        return False
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), ref_root])
    return True


if __name__ == "__main__":
    build(verbose=True)
    build_reference()
