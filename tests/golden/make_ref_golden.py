"""Generate tests/golden/ref_kernels.npz: outputs of the REFERENCE's own CUDA
kernels (cunusht/c/pointing.cu, cunusht/c/doubling.cu, built into
oracle/_ref by oracle/ref_build.py) on the seeded inputs of ref_cases.py.

Runs on a GPU with oracle/_ref present:
    python tests/golden/make_ref_golden.py [out.npz]
TEST INFRASTRUCTURE ONLY.  The fixture stores inputs and outputs, so the
parity test compares against it without the cubins."""
from __future__ import annotations

import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def _cases():
    spec = importlib.util.spec_from_file_location("ref_cases", os.path.join(HERE, "ref_cases.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def run_reference(cases):
    """{key: array} of inputs and reference outputs for every case."""
    import torch
    from oracle import ref_kernels as rk
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")
    out = {}
    for name in cases.POINTING:
        th, ph0, nph, ofs, dth, dph = cases.pointing_inputs(name)
        nring, npix = th.size, dth.size
        pad = lambda a, v: np.append(a, v)
        pt = torch.full((npix,), np.nan, dtype=torch.float64, device="cuda")
        pp = torch.full((npix,), np.nan, dtype=torch.float64, device="cuda")
        rk.pointing_lowmem(dev(pad(th, 0.0)), dev(pad(ph0, 0.0)), dev(pad(nph, 0)), dev(pad(ofs, npix)),
                           dev(dth), dev(dph), pt, pp, nring)
        for k, v in (("th", th), ("ph0", ph0), ("nph", nph), ("ofs", ofs),
                     ("dth", dth), ("dph", dph), ("pt", pt.cpu().numpy()), ("pp", pp.cpu().numpy())):
            out[f"pointing/{name}/{k}"] = v
    for name in cases.DOUBLING:
        for dt in (np.float64, np.float32):
            nt, nphi, cc, dm = cases.doubling_inputs(name, dt)
            tag = f"doubling/{name}/{np.dtype(dt).name}"
            o1 = torch.full(((2 * nt - 2) * nphi,), np.nan, dtype=dev(cc).dtype, device="cuda")
            rk.doubling_ring(dev(cc), nt, nphi, o1)
            o2 = torch.full(((2 * nt - 2) * nphi,), np.nan, dtype=dev(cc).dtype, device="cuda")
            rk.doubling_contig(dev(cc.T), nt, nphi, o2)                # theta-contiguous (nphi, nt) in
            o3 = torch.full((nt * nphi,), np.nan, dtype=dev(cc).dtype, device="cuda")
            rk.adjoint_doubling(dev(dm), nt, nphi, o3)
            out[tag + "/cc"] = cc
            out[tag + "/dm"] = dm
            out[tag + "/ring"] = o1.cpu().numpy().reshape(2 * nt - 2, nphi)
            out[tag + "/contig"] = o2.cpu().numpy().reshape(nphi, 2 * nt - 2)
            out[tag + "/adjoint"] = o3.cpu().numpy().reshape(nt, nphi)
    return out


if __name__ == "__main__":
    dst = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "ref_kernels.npz")
    data = run_reference(_cases())
    np.savez_compressed(dst, **data)
    print(f"wrote {dst}: {len(data)} arrays, {os.path.getsize(dst)} bytes")
