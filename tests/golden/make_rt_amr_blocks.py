"""Write the Rayleigh-Taylor refined pack's block list (rt2d_amr_blocks.json): level, origin,
size and face table of each of the 1440 leaf blocks, as generated by
apophis_gb300.amr.rt2d_amr().  tests/test_amr_oracle.py checks that the generator still
produces exactly this list."""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from apophis_gb300 import amr  # noqa: E402


def block_list():
    cfg, _ = amr.rt2d_amr()
    return {"base_nx": list(cfg.base_nx), "xmin": list(cfg.xmin), "xmax": list(cfg.xmax),
            "bc": [list(b) for b in cfg.bc], "ng": cfg.ng,
            "blocks": [{"level": B.level, "origin": list(B.origin), "nx": list(B.nx),
                        "face_kind": list(B.face_kind), "face_nbr": [list(n) for n in B.face_nbr]}
                       for B in cfg.blocks]}


if __name__ == "__main__":
    with open(os.path.join(HERE, "rt2d_amr_blocks.json"), "w") as f:
        json.dump(block_list(), f, separators=(",", ":"))
