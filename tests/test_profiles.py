"""The committed profile summaries: every bench.py command line they quote
uses options the benchmark has, and the traversal's traffic record (read by
the benchmark's roofline) parses."""
import os
import re
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench_options():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True,
                         text=True, check=True).stdout
    return set(re.findall(r"--[a-z][a-z0-9-]*", out))


def test_profile_commands_use_bench_options():
    opts = _bench_options()
    pdir = os.path.join(ROOT, "profiles")
    seen = 0
    for name in sorted(os.listdir(pdir)):
        if not name.endswith(".md"):
            continue
        text = open(os.path.join(pdir, name)).read()
        for block in re.findall(r"```\n(.*?)```", text, flags=re.S):
            cmd = block.replace("\\\n", " ")
            for m in re.finditer(r"python bench\.py((?:\s+--?[a-z][\w-]*(?:\s+[0-9]+)*)*)", cmd):
                for opt in re.findall(r"--[a-z][a-z0-9-]*", m.group(1)):
                    assert opt in opts, (name, opt)
                seen += 1
    assert seen >= 5  # the summaries quote their commands


def test_traversal_traffic_record():
    sys.path.insert(0, ROOT)
    import bench

    tpr = bench.ncu_traffic_per_ray()
    assert tpr is not None and 16.0 <= tpr < 2000.0  # at least the hit stores
    l2 = bench.ncu_l2()
    assert 0.0 < l2["lts__t_sector_hit_rate.pct"] <= 100.0
    r = bench.roofline(2.0e9, 1.0e-3, "model", "timed")
    assert r["bound"] == "hbm" and abs(r["achieved"] - 2000.0) < 1e-9 and r["frac"] > 0.0
