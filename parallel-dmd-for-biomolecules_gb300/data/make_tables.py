"""Writes prime20_tables.json: the PRIME20 parameter tables parsed from a
reference checkout (parameters/ and parametersep/ep19p_ha55a_weakhp.data,
the table code/inputinfo.f:282 reads) with dmdgb.params.

    python make_tables.py <reference>/parallel-dmd-PRIME20   (or set DMD_REFERENCE_DIR)
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from dmdgb.params import read_tables  # noqa: E402


def main(ref_root: str) -> None:
    t = read_tables(os.path.join(ref_root, "parameters"),
                    os.path.join(ref_root, "parametersep", "ep19p_ha55a_weakhp.data"))
    with open(os.path.join(HERE, "prime20_tables.json"), "w") as fh:
        json.dump(t.to_json(), fh, separators=(",", ":"))
        fh.write("\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["DMD_REFERENCE_DIR"])
