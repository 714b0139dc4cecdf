"""Reference gradient of the 128^3 adjoint workload (scenario.design_problem(): vacuum 128^3,
10-cell CPML, 32 x 32 x 16 design region of eps_r ~ U[1, 12], one 50-ohm source, Ez probe, 4000
steps) from the CPU oracle in FP64:

  * the FP64 discrete-adjoint gradient over the whole design region (oracle.fom_grad with the
    design-region history form), and J;
  * central differences of the FP64 oracle forward, h = 1e-3, at 16 seeded voxels.

    python tests/golden/make_adjoint_c4.py --out tests/golden/adjoint_c4.npz [--steps 4000] [--voxels 16]

Needs no GPU; takes tens of minutes on a few host cores (33 FP64 forwards of 8.4 G cell-updates
and one reverse sweep). tests/test_gpu_adjoint.py compares the GPU gradient with the file.
"""
import argparse
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from fdtd_gb300 import scenario as S  # noqa: E402

FD_SEED = 128  # voxel choice


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--voxels", type=int, default=16)
    ap.add_argument("--h", type=float, default=1e-3)
    a = ap.parse_args()
    d = S.design_problem(128, a.steps)
    sc = d.scenario
    e64 = d.eps.astype(np.float64)
    t0 = time.time()
    J, g = oracle.fom_grad(sc, d.probe, d.box, e64, box_history=True)
    print(f"J = {J:.9e}, adjoint {time.time() - t0:.0f} s", flush=True)
    rng = np.random.default_rng(FD_SEED)
    vox = [tuple(int(rng.integers(0, s)) for s in d.eps.shape) for _ in range(a.voxels)]
    fd = []
    for q, v in enumerate(vox):
        e1 = e64.copy(); e1[v] += a.h
        e2 = e64.copy(); e2[v] -= a.h
        f = (oracle.fom_grad(sc, d.probe, d.box, e1, grad=False) - oracle.fom_grad(sc, d.probe, d.box, e2, grad=False)) / (2 * a.h)
        fd.append(f)
        print(f"voxel {q} {v}: fd {f:.6e} adjoint {g[v]:.6e} rel {abs(g[v] - f) / abs(f):.2e} ({time.time() - t0:.0f} s)",
              flush=True)
    np.savez_compressed(a.out, steps=a.steps, h=a.h, J=J, grad=g, voxels=np.array(vox, dtype=np.int32),
                        fd=np.array(fd), box=np.array(d.box, dtype=np.int32), probe=np.array(d.probe, dtype=np.int32))
    print("wrote", a.out)


if __name__ == "__main__":
    main()
