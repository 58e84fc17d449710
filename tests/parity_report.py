"""Per-stage parity of the GPU path against the FP64 oracle, as a table.

    python tests/parity_report.py        (needs a GPU and the built library)

Runs the small Born (512^2 holograms, 128^2 fields, 256^3) and Rytov
(512^2, 128^2, 256^3, 40 rad phase) stacks of the parity tests through each
entry point and prints, per stage, the worst rel-L2 over the angles (or the
volume's), and the exact-match checks of the discrete outputs.
"""
from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import oracle  # noqa: E402
from mtd_transmission_gb300 import Context, Geometry  # noqa: E402
from tests.helpers import c64, oracle_cfg, rel_l2, small_case  # noqa: E402

CASES = (("Born", "plain_512_born", {}),
         ("Rytov", "rytov_1024", dict(ccd_roix=512, nxmax=64, circle_cx=128, circle_cy=128, dim_final=256)))


def run(name, workload, over, M=8):
    acq, _, d = small_case(workload, M=M, **over)
    cfg = oracle_cfg(acq)
    F, D = 2 * acq.nxmax, acq.dim_final
    holos = np.ascontiguousarray(d["holos"])
    spec = oracle.extract_stack(holos.astype(np.float64), cfg)
    fields, pos, dbg = oracle.fields(spec, cfg, d["mask"], debug=True)
    ref = oracle.reconstruction(fields, pos, cfg)
    rows = {}
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        sp = np.zeros((M, F, F), np.complex64)
        ctx.extract(holos, spectra_out=sp)
        rows["extraction (spectra)"] = max(rel_l2(sp[a], spec[a]) for a in range(M))
        fo = np.zeros((M, F, F), np.complex64)
        po = np.zeros(2 * M, np.int32)
        ph = np.zeros((M, F, F), np.float32)
        un = np.zeros_like(ph)
        am = np.zeros_like(ph)
        ctx.fields_debug(c64(spec), fields_out=fo, posspec_out=po, phase=ph, unwrapped=un, amp=am)
        rows["specular positions equal"] = bool(np.array_equal(po, pos.astype(np.int32)))
        rows["amplitude"] = max(rel_l2(am[a], dbg["amp"][a]) for a in range(M))
        rows["unwrapped phase"] = max(rel_l2(un[a], dbg["unwrap"][a]) for a in range(M))
        rows["fields (from oracle spectra)"] = max(rel_l2(fo[a], fields[a]) for a in range(M))
        re = np.zeros((D, D, D), np.float32)
        im = np.zeros_like(re)
        otf = np.zeros((D, D, D), np.uint8)
        cnt = np.zeros((D, D, D), np.uint32)
        ctx.reconstruct(c64(fields), pos.astype(np.int32), indice=re, absorption=im, otf=otf, counts=cnt)
        rows["hit counts equal"] = bool(np.array_equal(cnt, ref["counts"].astype(np.uint32)))
        rows["OTF mask equal"] = bool(np.array_equal(otf, ref["otf"]))
        rows["volume from oracle fields (index)"] = rel_l2(re, ref["indice"].real)
        rows["volume from oracle fields (absorption)"] = rel_l2(im, ref["indice"].imag)
        ctx.pipeline(holos, indice=re, absorption=im, counts=cnt)
        rows["end to end volume (index)"] = rel_l2(re, ref["indice"].real)
        rows["end to end volume (absorption)"] = rel_l2(im, ref["indice"].imag)
        rows["end to end hit counts equal"] = bool(np.array_equal(cnt, ref["counts"].astype(np.uint32)))
    return rows


def main():
    results = {name: run(name, wl, over) for name, wl, over in CASES}
    keys = list(next(iter(results.values())).keys())
    print("| stage | " + " | ".join(results) + " |")
    print("|---|" + "---|" * len(results))
    for k in keys:
        cells = []
        for name in results:
            v = results[name][k]
            cells.append(("yes" if v else "NO") if isinstance(v, bool) else f"{v:.2e}")
        print(f"| {k} | " + " | ".join(cells) + " |")


if __name__ == "__main__":
    main()
