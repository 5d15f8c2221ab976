"""Build the CPU oracle (test infrastructure).

  oracle/libupside_oracle.so   the CPU restatement (cpu_engine.cpp), any host
  oracle/_ref/libupside_ref.so the unmodified reference engine, built from the
                               reference checkout when it is present on an
                               x86-64 host (see ref_build/Makefile)
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_CSRC = os.path.join(HERE, "..", "upside2-md_gb300", "csrc")
# the reference checkout: $UPSIDE_REFERENCE, else a "reference" directory beside the repository
REF = os.environ.get("UPSIDE_REFERENCE", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def build_oracle():
    lib = os.path.join(HERE, "libupside_oracle.so")
    srcs = [os.path.join(HERE, "cpu_engine.cpp"), os.path.join(PKG_CSRC, "h5lite.cpp")]
    deps = srcs + [os.path.join(HERE, "cpu_engine.h"), os.path.join(PKG_CSRC, "h5lite.h")]
    if os.path.exists(lib) and all(os.path.getmtime(lib) > os.path.getmtime(d) for d in deps):
        return lib
    # no contraction into fused multiply-adds, so that the restatement
    # rounds alike on every host (aarch64 compilers contract by default)
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", PKG_CSRC, "-o", lib] + srcs
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode:
        raise RuntimeError("oracle build failed:\n" + r.stdout)
    return lib


def build_reference():
    """Reference engine oracle; None when the checkout is absent or the host is not x86-64."""
    if not os.path.isdir(os.path.join(REF, "src")) or platform.machine() not in ("x86_64", "AMD64"):
        return None
    r = subprocess.run(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref_build"), "REF=" + REF],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode:
        raise RuntimeError("reference oracle build failed:\n" + r.stdout[-4000:])
    return os.path.join(HERE, "_ref", "libupside_ref.so")


if __name__ == "__main__":
    print(build_oracle())
    print(build_reference())
