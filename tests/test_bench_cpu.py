"""bench.py on the CPU: the reference arm (the oracle's restatement on host threads) prints one
JSON line per workload and variant, named as the GPU arm names it; and the variants refuse
configs they do not apply to."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def oracle_built():
    r = subprocess.run([sys.executable, "-c", "import oracle.build as b; b.build()"], cwd=ROOT,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def run(*args):
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
           "--ref-seconds", "0.2", *args]
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)


@pytest.mark.parametrize("args, workload", [
    (("--config", "c2", "--variant", "window", "--scale", "0.002"),
     "affine-extend-window-band128-xdrop50-cigar"),
    (("--config", "c1", "--variant", "kslack", "--scale", "0.002"), "myers-infix-10k-cap-d+16"),
    (("--config", "c1", "--variant", "kdecoy", "--scale", "0.002"),
     "myers-global-10k-decoys-cap160"),
    (("--config", "c2", "--scale", "0.002", "--cigar", "0"), "affine-global-band128-score-20k"),
])
def test_reference_arm_variants(args, workload):
    r = run(*args)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["config"]["workload"] == workload
    assert d["value"] > 0 and d["unit"] == "GCUPS"
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_line_carries_the_contract_keys():
    """The keys a bench line must carry, with their types, on the reference arm's line."""
    r = run("--config", "c2", "--scale", "0.002")
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][0])
    for k, t in (("metric", str), ("value", float), ("unit", str), ("n_gpus", int),
                 ("steps", int), ("warmup", int), ("higher_is_better", bool),
                 ("scaling", str), ("dtype", str), ("data", str), ("config", dict),
                 ("e2e", dict), ("cpu_baseline", dict)):
        assert isinstance(d.get(k), t), (k, d.get(k))
    assert "vs_baseline" in d and "ms_per_step" in d
    assert d["impl"] == "reference" and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["unit"] == d["unit"] and d["e2e"]["value"] == d["value"]


def test_variant_of_another_config_is_refused():
    r = run("--config", "c3", "--variant", "window", "--scale", "0.002")
    assert r.returncode != 0
    assert "does not apply" in r.stderr
