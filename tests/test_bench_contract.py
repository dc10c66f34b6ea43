"""bench.py's JSON contract, checked on the CPU through its reference arm (the
oracle port on the host cores) and its configuration helpers."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_config_names_the_workload(F):
    sys.path.insert(0, ROOT)
    import bench
    for preset, batch in ((0, 4096), (1, 2048)):
        cfg = bench.config_of(F.params_preset(preset), batch)
        assert cfg["workload"].startswith("%d independent NAND-gate bootstraps" % batch)
        assert cfg["batch"] == batch and "l2" in cfg


def test_reference_arm_prints_one_json_line(F):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_loads_no_product_code():
    """The CPU reference arm makes its keys and inputs with the oracle alone:
    neither the product package nor libfheacc.so is loaded in its process."""
    code = (
        "import sys, types, json\n"
        "sys.argv = ['bench.py']\n"
        "import bench\n"
        "bench.run_reference(types.SimpleNamespace(preset=0, batch=64, warmup=1, steps=1, cpu_sample=2))\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libfheacc' not in maps, 'product library mapped'\n"
        "assert not any(m.startswith('3rd_gen_fhe_acc_gb300') for m in sys.modules), 'product package imported'\n"
        "print('clean')\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "clean" in r.stdout
