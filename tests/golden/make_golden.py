"""Generate tests/golden/oracle_golden.npz: small oracle outputs pinned as
regression fixtures (Morton codes, sort order, flattened tree, hits, pass
records, film) for seeded synthetic scenes. The reference itself publishes no
golden vectors and cannot be run here, so these pin the oracle across hosts
and over time. Run from the repository root:  python -m tests.golden.make_golden
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def compute(W, O):
    out = {}
    g0 = W.SceneGen(0, 0, (32, 32))
    o0 = O.OracleScene(g0.desc)
    e = o0.bvh_export()
    for k in ("codes", "sorted_prims", "nodes", "node_bounds"):
        out["c0_" + k] = e[k]
    L, w = o0.render(32, 32, 4)
    out["c0_film_L"] = L
    out["c0_film_w"] = w
    rec = o0.render_pass(1, 4, 0, 0, (8, 8, 16, 16), fields=["hit_prim", "L", "l_flags", "b_flags"])
    for k, v in rec.items():
        out["c0_rec_" + k] = v
    g1 = W.SceneGen(1, 0, (32, 32), level=4, rays=True)
    o1 = O.OracleScene(g1.desc)
    e1 = o1.bvh_export()
    out["c1_sorted_prims"] = e1["sorted_prims"]
    out["c1_nodes"] = e1["nodes"]
    out["c1_hits"] = o1.trace(g1.rays(), mode=0)
    return out


if __name__ == "__main__":
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle.build import build_oracle
    from woodenpbrengine_gb300.build import build_library

    build_library()
    build_oracle()
    import woodenpbrengine_gb300 as W
    from oracle import binding as O

    res = compute(W, O)
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **res)
    print({k: np.asarray(v).shape for k, v in res.items()})
