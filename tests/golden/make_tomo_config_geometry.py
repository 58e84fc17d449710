"""Writes tomo_config_geometry.json: the geometry that tdm_read_geom parses
from the reference's own configuration files (Tomo_config/recon.txt and
Tomo_config/config_manip.txt of madeba/MTD_transmission), so that tests on
machines without the reference tree run at that geometry.

    python tests/golden/make_tomo_config_geometry.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

FIELDS = ("ccd_roix", "nxmax", "circle_cx", "circle_cy", "dim_final", "born", "c_aber", "deroul", "volkov", "na",
          "n0", "lambda0", "f_tube", "f_obj", "tpcam", "rf", "coef_na_obj_limit")


def parse(root: str) -> dict:
    from mtd_transmission_gb300 import api
    g = api.read_geom(os.path.join(root, "Tomo_config", "recon.txt"),
                      os.path.join(root, "Tomo_config", "config_manip.txt"))
    return {k: getattr(g, k) for k in FIELDS}


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    out = os.path.join(HERE, "tomo_config_geometry.json")
    with open(out, "w") as f:
        json.dump(parse(root), f, indent=1)
        f.write("\n")
    print(out)
