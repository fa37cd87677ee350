"""Record the Result of run_simulation_b200 on the reference CLI's dev tier
(IFJ AIC-144, Markus 2 mm, the `dev` grid of examples/ifj_aic144/
run_markus_2mm.py) as tests/golden/b200_result_aic144_dev.npz.

Runs on a GB300 (the product has no CPU path). The reference's own writers
then consume this Result in tests/test_reference_integration.py, in a
container that has the reference checkout (which the GPU host does not).

    python tests/golden/make_b200_record.py [OUT.npz]
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE.parent))


def main():
    from goldens import make_config, pkg

    out = Path(sys.argv[1]) if len(sys.argv) > 1 else HERE / "b200_result_aic144_dev.npz"
    cfg = make_config("aic144_dev")
    res = pkg().run_simulation_b200(cfg, progress=False, return_fields=False)
    np.savez_compressed(out, time_s=res.time_s, f_t=res.f_t, ks=np.float64(res.ks), n_positive=res.n_positive,
                        n_negative=res.n_negative, injected_positive=res.injected_positive,
                        injected_negative=res.injected_negative, recombination=res.recombination,
                        track_density_xy=res.track_density_xy)
    print(f"{out}: k_s {res.ks:.10f}, {int(res.track_density_xy.sum())} tracks, {len(res.time_s)} steps")


if __name__ == "__main__":
    main()
