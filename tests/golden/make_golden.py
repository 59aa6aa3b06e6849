"""Writes the golden fixtures under tests/golden/ from the reference itself.

Run in a container where the reference checkout is present:

    python tests/golden/make_golden.py [--ref-root PATH] [--out-dir DIR]

1. ``element_matrices.json``: the four Maxima element matrices that the
   reference's own test hard-codes (Ke 8x8 and 24x24, Be 3x8 and 6x24,
   tests/test_bri17.cpp:344-356, :372-531, :547-552, :570-598), parsed from
   that file as text, with the fixture grids, material and tolerances of
   tests/test_bri17.cpp:319-333, :360, :535, :558, :604.
2. ``modal_ref.npz``: outputs of the reference header's own
   ``Hooke::modal_stiffness`` and ``Hooke::modal_strain_displacement``
   (include/bri17/bri17.hpp:212-292), compiled unmodified into
   oracle/_ref/libbri17_ref.so, over every frequency of several grids plus
   out-of-range and negative multi-indices; and the reference's
   ``get_cell_nodes`` tables.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


def default_ref_root() -> str:
    """The reference checkout this script reads: where oracle/Makefile
    reads it (BRI17_REF_ROOT overrides)."""
    from oracle import oracle as O
    return O.ref_root()


def parse_blocks(src: str, name: str):
    """Every ``<name> << v, v, ...;`` initializer in the source, in order."""
    out = []
    for m in re.finditer(name + r"\s*<<(.*?);", src, re.S):
        body = re.sub(r"//[^\n]*", "", m.group(1))
        vals = [float(v) for v in re.split(r"[,\s]+", body.strip()) if v]
        out.append(vals)
    return out


# Grids of the modal fixtures: the reference test grids plus larger,
# anisotropic and non-power-of-two grids of both dimensions.
MODAL_CASES = [
    dict(shape=[3, 4], L=[3.3000000000000003, 4.8], mu=5.6, nu=0.3),
    dict(shape=[3, 4, 5], L=[3.3000000000000003, 4.8, 6.5], mu=5.6, nu=0.3),
    dict(shape=[16, 12], L=[1.0, 1.0], mu=1.0, nu=0.3),
    dict(shape=[6, 10, 8], L=[1.0, 2.5, 0.75], mu=1.7, nu=0.45),
    dict(shape=[12, 9, 7], L=[1.0, 1.0, 0.125], mu=0.5, nu=0.1),
    dict(shape=[8, 8, 8], L=[1.0, 1.0, 1.0], mu=1.0, nu=0.25),
]


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=None)
    ap.add_argument("--out-dir", default=HERE,
                    help="where to write the fixtures (default: beside this script)")
    args = ap.parse_args(argv)
    if args.ref_root is None:
        args.ref_root = default_ref_root()
    out = args.out_dir
    test_src = os.path.join(args.ref_root, "tests", "test_bri17.cpp")
    with open(test_src) as f:
        src = f.read()
    ke = parse_blocks(src, "Ke")
    be = parse_blocks(src, "Be")
    assert len(ke) == 2 and len(be) == 2, (len(ke), len(be))
    assert len(ke[0]) == 64 and len(ke[1]) == 576, (len(ke[0]), len(ke[1]))
    assert len(be[0]) == 24 and len(be[1]) == 144, (len(be[0]), len(be[1]))
    spacing2, spacing3 = [1.1, 1.2], [1.1, 1.2, 1.3]
    shape2, shape3 = [3, 4], [3, 4, 5]
    # L = shape * spacing, computed with the same double products as
    # std::transform(..., std::multiplies()) at tests/test_bri17.cpp:326-333.
    L2 = [float(np.float64(n) * np.float64(s)) for n, s in zip(shape2, spacing2)]
    L3 = [float(np.float64(n) * np.float64(s)) for n, s in zip(shape3, spacing3)]
    golden = {
        "source": "tests/test_bri17.cpp (sbrisard/bri17), Maxima element matrices",
        "mu": 5.6,
        "nu": 0.3,
        "rtol": 1e-15,
        "atol": 1e-14,
        "imag_tol": 1e-14,
        "cases": [
            {"name": "2D stiffness matrix", "kind": "K", "dim": 2, "shape": shape2,
             "L": L2, "rows": 8, "cols": 8, "values": ke[0]},
            {"name": "3D stiffness matrix", "kind": "K", "dim": 3, "shape": shape3,
             "L": L3, "rows": 24, "cols": 24, "values": ke[1]},
            {"name": "2D strain-displacement matrix", "kind": "B", "dim": 2,
             "shape": shape2, "L": L2, "rows": 3, "cols": 8, "values": be[0]},
            {"name": "3D strain-displacement matrix", "kind": "B", "dim": 3,
             "shape": shape3, "L": L3, "rows": 6, "cols": 24, "values": be[1]},
        ],
    }
    with open(os.path.join(out, "element_matrices.json"), "w") as f:
        json.dump(golden, f, indent=1)

    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref",
                    f"REF_ROOT={args.ref_root}"], check=True, stdout=subprocess.DEVNULL)
    from oracle import oracle as O
    R = O.ref_lib()
    assert R is not None
    arrays = {}
    meta = []
    rng = np.random.default_rng(17)
    for ci, case in enumerate(MODAL_CASES):
        shape, L = case["shape"], case["L"]
        dim = len(shape)
        grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
        k_full = np.stack([g.reshape(-1) for g in grids], axis=1)
        k_out = rng.integers(-3 * max(shape), 3 * max(shape), size=(64, dim))
        k = np.ascontiguousarray(np.concatenate([k_full, k_out]), dtype=np.intc)
        n = k.shape[0]
        sa, sp = O._iarr(shape)
        La, Lp = O._darr(L)
        K = np.empty((n, dim * dim), dtype=np.complex128)
        B = np.empty((n, dim), dtype=np.complex128)
        R.ref_modal_stiffness_batch(dim, sp, Lp, case["mu"], case["nu"],
                                    k.ctypes.data_as(O._ip), n, K.ctypes.data_as(O._dp))
        R.ref_modal_strain_displacement_batch(dim, sp, Lp, case["mu"], case["nu"],
                                              k.ctypes.data_as(O._ip), n,
                                              B.ctypes.data_as(O._dp))
        size = int(np.prod(shape))
        nodes = np.empty((size, 1 << dim), dtype=np.intc)
        R.ref_all_cell_nodes(dim, sp, nodes.ctypes.data_as(O._ip))
        arrays[f"k_{ci}"] = k
        arrays[f"K_{ci}"] = K
        arrays[f"B_{ci}"] = B
        arrays[f"nodes_{ci}"] = nodes
        meta.append(case)
    np.savez_compressed(os.path.join(out, "modal_ref.npz"), **arrays)
    with open(os.path.join(out, "modal_ref.json"), "w") as f:
        json.dump({"source": "include/bri17/bri17.hpp (sbrisard/bri17) compiled "
                             "unmodified by oracle/Makefile, -O2 -ffp-contract=off",
                   "cases": meta}, f, indent=1)
    print("wrote", sorted(os.listdir(out)))


if __name__ == "__main__":
    main()
