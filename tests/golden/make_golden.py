"""Generate the golden fixtures under tests/golden from the reference checkout.

Run where the reference checkout is present (it is not on the GPU machines):
    python tests/golden/make_golden.py <reference checkout>
or with MPM_REFERENCE_ROOT naming the checkout.
Writes:
  ref_linalg.json  — the matrices and tolerances of the reference's own tests
                     (tests/test_linalg.cu: TestPolar.*, TestDevicePolar.Basic,
                     TestDeterminant.Identity), read from the test source as text.
  ref_svd.npz      — seeded 3x3 matrices and the outputs of the reference's own
                     include/svd3_cuda.h, compiled for the host (oracle/_ref).
  ref_substep.npz  — (when oracle/_ref/libref_substep.so is built) small seeded
                     particle states advanced by the reference's own policy headers.
  ref_mesh.npz     — (when oracle/_ref/libref_mesh.so is built) distance fields of
                     seeded particle sets from the reference's include/mesh_builder.h.
"""
import ctypes
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402

REF = None  # the reference checkout, set by main() from argv[1] or MPM_REFERENCE_ROOT


def linalg_vectors():
    src = open(os.path.join(REF, "tests", "test_linalg.cu")).read()
    mats = []
    for m in re.finditer(r"M << ([^;]+);", src):
        vals = [float(t) for t in m.group(1).split(",")]
        mats.append(vals)
    tols = sorted({float(t) for t in re.findall(r"ASSERT_LT\(\w+, ([0-9.e-]+)\)", src)})
    return {"source": "tests/test_linalg.cu", "matrices": mats, "tolerances": tols,
            "det_identity": 1.0}


def svd_vectors():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_svd.so"))
    rng = np.random.default_rng(1234)
    A = [rng.standard_normal((96, 3, 3)),
         np.eye(3) + 0.05 * rng.standard_normal((96, 3, 3)),
         np.eye(3)[None] * rng.uniform(0.5, 1.5, (32, 1, 1)),
         rng.standard_normal((32, 3, 3)) * np.array([1, 1, 0])[None, :, None]]
    A = np.concatenate(A, 0).astype(np.float32)
    lin = linalg_vectors()
    extra = np.array([np.array(m, np.float32).reshape(3, 3) for m in lin["matrices"]])
    A = np.ascontiguousarray(np.concatenate([A, extra], 0))
    n = A.shape[0]
    U = np.zeros_like(A)
    V = np.zeros_like(A)
    s = np.zeros((n, 3), np.float32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    lib.ref_svd(ctypes.c_int64(n), P(A), P(U), P(s), P(V))
    return {"A": A, "U": U, "s": s, "V": V}


def main():
    global REF
    REF = obuild.reference_root(sys.argv[1] if len(sys.argv) > 1 else None)
    if REF is None:
        raise SystemExit("reference checkout not given (argv[1] or MPM_REFERENCE_ROOT); fixtures unchanged")
    obuild.build_oracle()
    built = obuild.build_ref(REF)
    if not built:
        raise SystemExit("reference libraries not built; fixtures unchanged")
    with open(os.path.join(HERE, "ref_linalg.json"), "w") as f:
        json.dump(linalg_vectors(), f, indent=1)
    np.savez_compressed(os.path.join(HERE, "ref_svd.npz"), **svd_vectors())
    sub = os.path.join(ROOT, "oracle", "_ref", "libref_substep.so")
    if os.path.exists(sub):
        sys.path.insert(0, HERE)
        import ref_substep_vectors

        np.savez_compressed(os.path.join(HERE, "ref_substep.npz"), **ref_substep_vectors.make(sub))
    mesh = os.path.join(ROOT, "oracle", "_ref", "libref_mesh.so")
    if os.path.exists(mesh):
        sys.path.insert(0, HERE)
        import ref_mesh_vectors

        np.savez_compressed(os.path.join(HERE, "ref_mesh.npz"), **ref_mesh_vectors.make(mesh))
    print("golden fixtures written")


if __name__ == "__main__":
    main()
