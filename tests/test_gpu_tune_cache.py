"""The autotuner's on-disk cache of launch shapes ($NLC_TUNE_CACHE): a plan of a tuned size times
its candidate shapes once and records the winner and its step time; a later process with the same
device, model, variant, chain length and copies bucket takes the shape from the file without a
single tuning launch.  Lines that do not parse are ignored; NLC_TUNE_CACHE=off writes no file.
Each case runs in a fresh process, since the process also keeps the shapes in memory."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# DNKG, 128 sites, 1024 chains: 131072 sites, above the size from which shapes are timed
SCRIPT = f'''
import json, sys
sys.path.insert(0, {ROOT!r})
import nlchains_gb300 as nlc
n0 = nlc.kernel_launches()
plan = nlc.Plan(nlc.Model("DNKG", 128, 1024, 0.05, m=1.0, beta=1.0))
print(json.dumps({{"launches": nlc.kernel_launches() - n0, "shape": plan.shape()}}))
'''


def plan_in_new_process(env):
    r = subprocess.run([sys.executable, "-c", SCRIPT], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_tuned_shape_comes_from_the_cache_file(gpu, tmp_path):
    cache = tmp_path / "shapes.tsv"
    env = dict(os.environ, NLC_TUNE_CACHE=str(cache))
    first = plan_in_new_process(env)
    assert first["launches"] > 0, "the first plan times its candidate shapes"
    lines = cache.read_text().splitlines()
    assert len(lines) == 1
    fields = lines[0].split("\t")
    assert len(fields) == 9 and int(fields[3]) == 128 and int(fields[4]) == 10   # n, copies bucket floor(log2 1024)
    assert float(fields[8]) > 0, "the step time feeds the rounds per launch"
    second = plan_in_new_process(env)
    assert second["launches"] == 0 and second["shape"] == first["shape"]
    with open(cache, "a") as f:
        f.write("not a shape line\n")
    third = plan_in_new_process(env)
    assert third["launches"] == 0 and third["shape"] == first["shape"]
    assert len(cache.read_text().splitlines()) == 2, "a cache hit appends nothing"


def test_cache_off_writes_no_file(gpu, tmp_path):
    env = dict(os.environ, NLC_TUNE_CACHE="off", HOME=str(tmp_path), XDG_CACHE_HOME=str(tmp_path / "xdg"))
    r = plan_in_new_process(env)
    assert r["launches"] > 0
    assert not list(tmp_path.rglob("shapes.tsv"))
