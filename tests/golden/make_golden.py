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
    # textured metal (scene config 5) and the Sampled64 film
    g5 = W.SceneGen(5, 0, (24, 16))
    o5 = O.OracleScene(g5.desc)
    out["c5_film_L"], out["c5_film_w"] = o5.render(24, 16, 2)
    out["c0_spectral_L"], _ = o0.render_spectral(32, 32, 1, 0, 0)
    # MIP pyramid and both texture samplers on a small odd-sized texture
    rng = np.random.default_rng(9)
    tex = rng.random((12, 20, 3), dtype=np.float32)
    for i, lv in enumerate(O.texture_levels(tex)):
        out["tex_level%d" % i] = lv
    fps = np.concatenate([rng.uniform(0.0, 1.0, (16, 2)), rng.normal(0.0, 0.05, (16, 4))], axis=1)
    out["tex_aniso"] = np.stack([O.texture_eval(tex, fp) for fp in fps])
    out["tex_iso"] = np.stack([O.texture_eval(tex, fp, isotropic=True) for fp in fps])
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
