"""Build recipe for the oracle (test infrastructure).

* ``libmpm_oracle.so`` — the C++ restatements of the reference substep, of particle
  seeding and of surface reconstruction (always).
* ``_ref/libref_svd.so`` — the reference's own ``include/svd3_cuda.h`` compiled
  for the host from where it lies in the reference checkout, through
  ``ref_shim/`` (host definitions of the three CUDA rounding intrinsics it uses).
  Built only when the reference checkout is given: the ``ref_root`` argument of
  :func:`build_ref`, else the ``MPM_REFERENCE_ROOT`` environment variable; without
  either it is skipped with a message.  Nothing from the reference is copied into
  the repository.
* ``_ref/libref_substep.so`` — the reference's own policy headers
  (TransferScheme.h, MaterialModel.cuh, InterpolationKernel.cuh, types.h,
  svd3_cuda.h) compiled for the host against the project-written Eigen subset in
  ``ref_shim/``, driven by the loop skeleton in ``ref_substep.cpp``.
* ``_ref/libref_mesh.so`` — the reference's own ``include/mesh_builder.h`` (its
  distance field) compiled for the host against the same Eigen subset plus the
  ``boost::multi_array`` and declaration-only libigl stand-ins in ``ref_shim/``,
  driven by ``ref_mesh.cpp``; no OpenMP, so its particle loop runs sequentially.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def _run(cmd):
    subprocess.run(cmd, check=True)


def build_oracle(force: bool = False) -> str:
    out = os.path.join(HERE, "libmpm_oracle.so")
    src = os.path.join(HERE, "mpm_oracle.cpp")
    seed = os.path.join(HERE, "seed_oracle.cpp")
    surface = os.path.join(HERE, "surface_oracle.cpp")
    hdr = os.path.join(HERE, "mpm_oracle.h")
    srcs = (src, seed, surface)
    if force or not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(f) for f in srcs + (hdr,)):
        tmp = out + ".tmp"
        _run(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
              "-o", tmp, *srcs])
        os.replace(tmp, out)
    return out


def reference_root(ref_root=None):
    """The reference checkout: the argument, else MPM_REFERENCE_ROOT; None when neither
    names a checkout (a directory holding include/svd3_cuda.h)."""
    root = ref_root or os.environ.get("MPM_REFERENCE_ROOT")
    if root and os.path.isfile(os.path.join(root, "include", "svd3_cuda.h")):
        return root
    return None


def build_ref(ref_root=None, force: bool = False) -> list:
    """Compile the reference-derived host libraries into oracle/_ref from the reference
    checkout (``ref_root`` or MPM_REFERENCE_ROOT). Returns the list of built paths;
    empty, with a message, when no checkout is given."""
    REF_ROOT = reference_root(ref_root)
    if REF_ROOT is None:
        print("oracle/_ref not built: no reference checkout given (pass ref_root or set MPM_REFERENCE_ROOT)")
        return []
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    inc = os.path.join(REF_ROOT, "include")
    shim = os.path.join(HERE, "ref_shim")
    built = []
    for name, src in (("libref_svd.so", "ref_svd.cpp"), ("libref_substep.so", "ref_substep.cpp"),
                      ("libref_mesh.so", "ref_mesh.cpp")):
        srcp = os.path.join(HERE, src)
        if not os.path.exists(srcp):
            continue
        out = os.path.join(outdir, name)
        deps = [srcp] + [os.path.join(d, f) for d, _, fs in os.walk(shim) for f in fs]
        if force or not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(d) for d in deps):
            tmp = out + ".tmp"
            # The shim directory comes first so its cuda.h / cuda_runtime.h / Eigen stand-ins
            # are found before any system header of the same name.
            _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                  "-I", shim, "-I", inc, "-I", os.path.join(REF_ROOT, "src"), "-o", tmp, srcp])
            os.replace(tmp, out)
        built.append(out)
    return built


if __name__ == "__main__":
    import sys

    print(build_oracle(force=True))
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
