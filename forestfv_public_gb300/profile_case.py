"""A profiler target: the FP32-flux form on the medium wall mesh (0.41 M cells, levels 4-7)
stepped `steps` times with one form of the flux, so that an ncu capture can skip the
launches of the early steps and measure a launch of the developed flow.

  python -m forestfv_public_gb300.profile_case [steps] [reference|consistent] [infer]

Each time step launches the FP32-flux stage kernels twice (RK2); launch k of a kernel belongs
to step k // 2.  With `infer`, the learned indicator (random weights, normalised on the
state) then marks the developed state three times: fields + the fused tcgen05 inference,
launches 0-2 of mlp_infer_tc."""
from __future__ import annotations

import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main() -> None:
    import bench
    from forestfv_public_gb300 import Solver
    steps = int(sys.argv[1]) if len(sys.argv) > 1 else 30
    form = sys.argv[2] if len(sys.argv) > 2 else "consistent"
    mesh, S0, dt, _, kw, _, _ = bench.wl_config3(medium=True)
    s = Solver(precision=1, flux_form=bench.FLUX_FORMS[form], **kw)
    s.set_mesh(mesh)
    s.upload_state(S0)
    t0 = time.perf_counter()
    s.step(dt, steps)
    print(f"{mesh.n} cells, {steps} steps of the FP32-flux form ({form} flux) in "
          f"{time.perf_counter() - t0:.3f} s")
    if len(sys.argv) > 3 and sys.argv[3] == "infer":
        import numpy as np
        import torch
        from .indicator import Indicator
        ind = Indicator(seed=3)
        F = ind.fields(s).cpu().numpy().astype(np.float64)
        ind.set_norm(F.mean(axis=1), F.std(axis=1) + 1e-3)
        marks = torch.zeros(mesh.n, dtype=torch.uint8, device=f"cuda:{s.device}")
        for _ in range(3):
            ind.mark(s, 0.5, marks, True)
        s.sync()
        print(f"{int(marks.sum())} cells marked")
        ind.close()
    s.close()


if __name__ == "__main__":
    main()
