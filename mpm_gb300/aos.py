"""The reference's AoS particle record, for callers that hold reference-layout data.

``MLS_APIC_Particle`` (include/TransferScheme.h:46-54 on ParticleBase,
include/types.h:24-35) is 104 bytes with Eigen's fixed-size (4-byte aligned,
column-major) members: u8 material_type, 3 pad bytes, Vec x, Vec v, Mat F,
Mat C, real Jp.
"""
import numpy as np

RECORD = np.dtype([("material_type", "u1"), ("pad", "u1", 3), ("x", "<f4", 3), ("v", "<f4", 3),
                   ("F", "<f4", 9), ("C", "<f4", 9), ("Jp", "<f4")])
assert RECORD.itemsize == 104


def pack(state: dict) -> np.ndarray:
    """SoA state (row-major 3x3) -> bytes of n reference records."""
    n = int(np.asarray(state["x"]).shape[0])
    r = np.zeros(n, RECORD)
    r["material_type"] = np.asarray(state.get("mat", np.zeros(n)), np.uint8)
    r["x"] = np.asarray(state["x"], np.float32)
    r["v"] = np.asarray(state.get("v", np.zeros((n, 3))), np.float32)
    F = np.asarray(state.get("F", np.tile(np.eye(3), (n, 1, 1))), np.float32).reshape(n, 3, 3)
    C = np.asarray(state.get("C", np.zeros((n, 3, 3))), np.float32).reshape(n, 3, 3)
    r["F"] = F.transpose(0, 2, 1).reshape(n, 9)  # column-major
    r["C"] = C.transpose(0, 2, 1).reshape(n, 9)
    r["Jp"] = np.asarray(state.get("Jp", np.ones(n)), np.float32)
    return r.view(np.uint8).reshape(-1)


def unpack(buf: np.ndarray) -> dict:
    r = np.ascontiguousarray(buf).view(RECORD)
    n = r.shape[0]
    return {"x": r["x"].copy(), "v": r["v"].copy(),
            "F": r["F"].reshape(n, 3, 3).transpose(0, 2, 1).copy(),
            "C": r["C"].reshape(n, 3, 3).transpose(0, 2, 1).copy(),
            "Jp": r["Jp"].copy(), "mat": r["material_type"].copy()}
