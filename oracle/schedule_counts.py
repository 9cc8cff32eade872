"""Block-solves and waves of the reference's own gHCM schedule on the
benchmark fields, from the oracle's CPU restatement (ghcm_oracle_hcm:
src/eikonal_hcm.cpp:186-482 with the systolic kernel,
data/eikonal_ghcm_systolic.cl:8-175), with how far each result ends from the
reference FIM's fixed point. Test infrastructure: it runs only the oracle.

    python -m oracle.schedule_counts            # prints one JSON object per field
"""
from __future__ import annotations

import json
import time

from ghcm_gb300 import fields
from oracle.oracle import Oracle, build, rel_diff

FIELDS = (
    # name, generator, tile, n, work-group lanes (the reference runs one work-group of WG lanes per tile)
    ("ring7_256 (C1)", lambda: fields.ring7_small(seed=1), 8, 64, 64),
    ("ring7_4096 (C2)", lambda: fields.ring7_large(1), 16, 256, 256),
    ("noise_4096_16src (C3)", lambda: fields.value_noise(4096, seed=1, base_period=512.0, sources=16), 16, 1024, 256),
)


def main() -> None:
    build(with_reference=False)
    o = Oracle()
    for name, make, block, n, wg in FIELDS:
        speed, seeds = make()
        cost = fields.cost_from_speed(speed)
        t0 = time.perf_counter()
        out, solves, waves = o.hcm(cost, seeds, block=block, max_jobs=n, eps=1e-5, wg=wg)
        secs = time.perf_counter() - t0
        fim = o.fim(cost, seeds, 1e-5)[0]
        print(json.dumps({"field": name, "block": block, "n": n, "work_group": wg, "block_solves": int(solves),
                          "waves": int(waves), "max_rel_vs_fim": rel_diff(out, fim),
                          "residual": o.residual(cost, out), "cpu_s": round(secs, 1)}), flush=True)


if __name__ == "__main__":
    main()
