"""Copies the reference's DCT-unwrap debug dumps into tests/golden as .npy fixtures.

The reference ships float32 little-endian dumps of its DCT unwrapping chain
(cTDM/src.256.256.raw -> Laplace -> DCT -> DCT2 -> IDCT; written by the
commented DeviceMemOutDCT calls in cTDM/DCT_Unwrapping.cu:35-55).  They are the
only reference-produced golden vectors for this path.  Run once where the
reference tree is available:  python tests/golden/make_golden.py <reference root>
"""
import hashlib
import json
import os
import sys

import numpy as np

NAMES = ["src", "Laplace", "DCT", "DCT2", "IDCT"]


def main(root):
    here = os.path.dirname(os.path.abspath(__file__))
    manifest = {}
    for name in NAMES:
        path = os.path.join(root, "cTDM", f"{name}.256.256.raw")
        raw = open(path, "rb").read()
        arr = np.frombuffer(raw, dtype="<f4").reshape(256, 256)
        np.save(os.path.join(here, f"dct_chain_{name}.npy"), arr)
        manifest[name] = {"source": f"cTDM/{name}.256.256.raw", "sha256": hashlib.sha256(raw).hexdigest(),
                          "shape": [256, 256], "dtype": "float32"}
    with open(os.path.join(here, "dct_chain_manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference root (the y-h-Lin/cTDM checkout)>")
    main(sys.argv[1])
