"""bench.py's reference arm on CPU: it runs the oracle's FP32 OpenMP port of the reference
kernels over W untimed and exactly K timed frames of the workload our arm times, reports a
finite ms_per_step and our arm's config dict, and never loads libpbd.so."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_times_k_frames_without_the_library():
    code = ("import sys, bench; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'dam_break_32k', "
            "'--steps', '2', '--warmup', '3']; bench.main(); "
            "print('LIBPBD_MAPPED', 'libpbd.so' in open('/proc/self/maps').read())")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600,
                         env={**os.environ, "OMP_NUM_THREADS": "4"})
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    assert lines[-1] == "LIBPBD_MAPPED False"
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 3
    assert line["ms_per_step"] > 0 and line["value"] > 0
    assert line["value"] == line["cpu_baseline"]["value"] == line["e2e"]["value"]
    assert line["config"]["workload"] == "dam_break_32k" and line["config"]["particles"] == 32768
    assert "frames 4-5" in line["cpu_baseline"]["sample"]


def test_reference_and_our_arm_share_the_config_dict():
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "pbd-simulation-framework-cuda_gb300"))
    import bench
    import pbd
    import scenes
    for name in ("fluid_1m", "fluid_1m_dense"):
        p_lib, pos, _, _ = bench.build_workload(pbd, scenes, name)
        p_orc, pos2, _, _ = bench.oracle_params(scenes, name)
        assert bytes(p_lib) == bytes(p_orc)
        assert bench.workload_config(name, p_lib, len(pos), 1) == bench.workload_config(name, p_orc, len(pos2), 1)
