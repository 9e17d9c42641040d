"""Generates the golden fixtures of this directory from the reference's own
test data (carstenbauer/dqmc `test/data/O3.jld` and `test/data/linalg.jld`).

Run with the path of a checkout of the reference, as an argument or in the
environment variable DQMC_REFERENCE:

    python tests/golden/make_golden.py <path-to-carstenbauer-dqmc>

Only datasets that do not depend on Julia's global RNG stream are kept (the
reference draws the others after `Random.seed!` with Julia <= 1.6's dSFMT,
which cannot be reproduced here).  The literal known answers that the
reference's test files spell out (boson action values, chi_static, Binder
factors, checkerboard corners, neighbour tables) are stored beside them, each
with the test-file line it comes from.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import scipy.sparse as sps

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from jld_reader import load_jld  # noqa: E402

O3_KEYS = [
    # RNG-independent datasets used by test/tests_O3.jl
    "randconf",                                   # :3
    "nob_chkr_hop1", "nob_chkr_hop2", "nob_chkr_hop_inv1", "nob_chkr_hop_inv2",            # :98-101
    "nob_chkr_hop_half1", "nob_chkr_hop_half2", "nob_chkr_hop_half_inv1", "nob_chkr_hop_half_inv2",  # :103-106
    "nob_chkr_mu", "nob_chkr_mu_half", "nob_chkr_mu_inv", "nob_chkr_mu_half_inv",           # :108-111
    "nob_eVplus", "nob_eVminus", "nob_eVexpop",   # :156-163
    "Ul", "Dl", "Tl", "Ur", "Dr", "Tr", "greens",  # :217-227 (calculate_greens KAT)
    "chi_dyn",                                    # tests_O3_measurements.jl:4
]
LINALG_KEYS = ["B_QR_U", "B_QR_D", "B_QR_T"]   # tests_linalg.jl:26-28, 105-113

# literal known answers written in the reference's test files
LITERALS = {
    "boson_action_randconf": 75.57712964980982,             # tests_O3.jl:51 (lambda .5, r 2, c 3, u 1)
    "boson_action_diff_site3_slice10": 0.015453643701304112,  # tests_O3.jl:52
    "boson_action_randconf_edrun": 16.348917129437076,      # tests_O3.jl:56
    "boson_action_diff_site3_slice10_edrun": 0.014491910524600016,  # tests_O3.jl:57
    "chi_static_randconf": 12.420575691388407,               # tests_O3_measurements.jl:5
    "binder_m2": 0.7762859807117749,                         # tests_O3_measurements.jl:6
    "binder_m4": 0.6026199238496421,
    "msafe_maxD": 5.8846316709257896e16,                     # tests_linalg.jl:111
    "msafe_minD": 1.9123571535539083e-24,                    # tests_linalg.jl:112
}
NEW_OP = np.array([0.370422, 0.797014, 0.956094])           # tests_O3.jl:52
EXPOP_OP = np.array([0.130018, 0.792039, 0.683411])         # tests_O3.jl:163
CORNERS_A = np.array([1, 3, 9, 11])                          # tests_O3.jl:96 (1-based)
CORNERS_B = np.array([6, 8, 14, 16])
NEIGHBORS_L4 = np.array([[2, 3, 4, 1, 6, 7, 8, 5, 10, 11, 12, 9, 14, 15, 16, 13],     # tests_O3.jl:268-271
                         [5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 1, 2, 3, 4],
                         [4, 1, 2, 3, 8, 5, 6, 7, 12, 9, 10, 11, 16, 13, 14, 15],
                         [13, 14, 15, 16, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12]])
TIME_NEIGHBORS_M10 = np.array([[2, 3, 4, 5, 6, 7, 8, 9, 10, 1],                  # tests_O3.jl:272
                               [10, 1, 2, 3, 4, 5, 6, 7, 8, 9]])


def jld_layout(path):
    """Encodings of the reference's JLD file that an output writer must match:
    the 512-byte user block, the superblock's version and size fields, the
    datatype messages of a Float64 array (`randconf`), an Int64 scalar
    (`_creator/WORD_SIZE`) and a UInt32 scalar (`_creator/JULIA_MAJOR`), and the
    member names of `_creator`."""
    from jld_reader import _Reader
    r = _Reader(path)
    root = r.links(r.root)
    creator = r.links(root["_creator"])

    def dtype_msg(addr):
        for mtype, _, data in r.messages(addr):
            if mtype == 0x03:
                return np.frombuffer(bytes(data), dtype=np.uint8)
        raise KeyError("no datatype message")

    d = r.d
    return {
        "jld_userblock": np.frombuffer(d[:512], dtype=np.uint8),
        "jld_superblock_head": np.frombuffer(d[r.base:r.base + 24], dtype=np.uint8),
        "jld_dt_float64_array": dtype_msg(root["randconf"]),
        "jld_dt_int64_scalar": dtype_msg(creator["WORD_SIZE"]),
        "jld_dt_uint32_scalar": dtype_msg(creator["JULIA_MAJOR"]),
        "jld_creator_names": np.array(sorted(creator)),
    }


def main(ref_root):
    o3 = load_jld(os.path.join(ref_root, "test", "data", "O3.jld"))
    la = load_jld(os.path.join(ref_root, "test", "data", "linalg.jld"))
    out = {}
    for k in O3_KEYS:
        v = o3[k]
        if isinstance(v, Exception):
            raise v
        out[k] = v.toarray() if sps.issparse(v) else np.asarray(v)
    for k in LINALG_KEYS:
        out[k] = np.asarray(la[k])
    for k, v in LITERALS.items():
        out["lit_" + k] = np.array(v)
    out["lit_new_op"] = NEW_OP
    out["lit_expop_op"] = EXPOP_OP
    out["lit_corners_A"] = CORNERS_A
    out["lit_corners_B"] = CORNERS_B
    out["lit_neighbors_L4"] = NEIGHBORS_L4
    out["lit_time_neighbors_M10"] = TIME_NEIGHBORS_M10
    out.update(jld_layout(os.path.join(ref_root, "test", "data", "O3.jld")))
    path = os.path.join(HERE, "o3_reference_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DQMC_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <path-to-carstenbauer-dqmc> (or set DQMC_REFERENCE)")
    main(ref)
