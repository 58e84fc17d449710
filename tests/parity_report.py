"""Per-stage parity of the GPU path against the FP64 oracle, as a table.

    python tests/parity_report.py          (needs a GPU and the built library)
    python tests/parity_report.py --full   (the two large workloads at full size)

Runs the small Born (512^2 holograms, 128^2 fields, 256^3) and Rytov
(512^2, 128^2, 256^3, 40 rad phase) stacks of the parity tests through each
entry point and prints, per stage, the worst rel-L2 over the angles (or the
volume's), and the exact-match checks of the discrete outputs.

--full runs rytov_1024 (600 x 1024^2, 256^2 fields, 512^3) and large_2048
(1000 x 2048^2, 512^2 fields, 1024^3) at full size: the per-angle stages on
3 sampled angles against the oracle, the volume stage against the oracle
from the GPU's fields of every angle at 512^3, and at 1024^3 (whose FP64
volume does not fit in host memory here) the dot-product mismatch of the
forward operator and its adjoint over every cap.
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


def run_full(workload):
    import torch
    from tests import simul
    from tests.test_gpu_full_size import _dot_product
    acq, ph, seed = simul.workload(workload)
    data = simul.holograms(acq, ph, seed=seed, device="cuda")
    holos = data["holos"].contiguous()
    mask = np.ascontiguousarray(data["mask"].cpu().numpy())
    if int((mask[::5, ::5] > 45).sum()) <= 9:
        mask = None  # no background on the fit grid: the unit mask, the reference's default
    del data
    torch.cuda.empty_cache()
    M, D, F = acq.nb_holo, acq.dim_final, 2 * acq.nxmax
    cfg = oracle_cfg(acq)
    oracle.set_threads(os.cpu_count() or 1)
    sample = [0, M // 2, M - 1]
    hs = np.stack([holos[a].cpu().numpy() for a in sample])
    spec = oracle.extract_stack(hs.astype(np.float64), cfg)
    fields, pos, dbg = oracle.fields(spec, cfg, mask, debug=True)
    S = len(sample)
    rows = {}
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        ctx.set_mask(mask)
        sp = np.zeros((S, F, F), np.complex64)
        ctx.extract(np.ascontiguousarray(hs), spectra_out=sp)
        rows["extraction (spectra)"] = max(rel_l2(sp[i], spec[i]) for i in range(S))
        fo = np.zeros((S, F, F), np.complex64)
        po = np.zeros(2 * S, np.int32)
        phs = np.zeros((S, F, F), np.float32)
        un = np.zeros_like(phs)
        am = np.zeros_like(phs)
        ctx.fields_debug(c64(spec), fields_out=fo, posspec_out=po, phase=phs, unwrapped=un, amp=am)
        rows["specular positions equal"] = bool(np.array_equal(po, pos.astype(np.int32)))
        rows["amplitude"] = max(rel_l2(am[i], dbg["amp"][i]) for i in range(S))
        rows["unwrapped phase"] = max(rel_l2(un[i], dbg["unwrap"][i]) for i in range(S))
        rows["fields (from oracle spectra)"] = max(rel_l2(fo[i], fields[i]) for i in range(S))
        gspec = torch.empty((M, F, F), dtype=torch.complex64, device="cuda")
        ctx.extract(holos, spectra_out=gspec)
        gf = torch.empty((M, F, F), dtype=torch.complex64, device="cuda")
        gpos = np.zeros(2 * M, np.int32)
        ctx.fields(gspec, fields_out=gf, posspec_out=gpos)
        del gspec
        if D <= 512:
            vol = lambda dt: np.zeros((D, D, D), dt)  # noqa: E731
            re, im, cnt = vol(np.float32), vol(np.float32), vol(np.uint32)
            ctx.reconstruct(gf, gpos, indice=re, absorption=im, counts=cnt)
            ref = oracle.reconstruction(gf.cpu().numpy(), gpos.astype(np.float64), cfg, want_otf=False)
            rows["hit counts equal (all angles)"] = bool(np.array_equal(cnt, ref["counts"].astype(np.uint32)))
            rows["volume from GPU fields (index)"] = rel_l2(re, ref["indice"].real)
            rows["volume from GPU fields (absorption)"] = rel_l2(im, ref["indice"].imag)
            rows["forward/adjoint dot-product mismatch"] = None
        else:
            rows["hit counts equal (all angles)"] = None
            rows["volume from GPU fields (index)"] = None
            rows["volume from GPU fields (absorption)"] = None
            rows["forward/adjoint dot-product mismatch"] = _dot_product(ctx, M, D, F, gpos)
    return rows


def cell(v):
    if v is None:
        return "—"
    return ("yes" if v else "NO") if isinstance(v, bool) else f"{v:.2e}"


def main():
    if "--full" in sys.argv:
        results = {wl: run_full(wl) for wl in ("rytov_1024", "large_2048")}
    else:
        results = {name: run(name, wl, over) for name, wl, over in CASES}
    keys = list(next(iter(results.values())).keys())
    print("| stage | " + " | ".join(results) + " |")
    print("|---|" + "---|" * len(results))
    for k in keys:
        print(f"| {k} | " + " | ".join(cell(results[name][k]) for name in results) + " |")


if __name__ == "__main__":
    main()
