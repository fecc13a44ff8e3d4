"""The step driven from C++ through the C ABI alone (examples/dam_break.cpp, the reference's
Simulation::step loop) gives the same state, bit for bit, as the Python binding on the same
parameters and spawn lattice."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "pbd-simulation-framework-cuda_gb300", "examples", "dam_break")


@pytest.mark.gpu
@pytest.mark.parametrize("vort,visc", [(0.0, 0.0), (0.0005, 0.01)])
def test_cpp_host_matches_the_python_binding(need_gpu, pbd, scenes, tmp_path, vort, visc):
    params = scenes.workload_params(pbd, 32, 1000.0, vorticity=vort, viscosity=visc)
    params.lambda_epsilon = 0.1
    (tmp_path / "params.bin").write_bytes(bytes(params))
    nx, ny, nz, sp, frames = 12, 10, 12, "0.9", 20
    out = tmp_path / "state.bin"
    r = subprocess.run([EXE, "--params", str(tmp_path / "params.bin"), "--lattice", str(nx), str(ny), str(nz), sp,
                        "--frames", str(frames), "--out", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert f"{nx * ny * nz} particles, {frames} frames" in r.stdout
    got = np.fromfile(out, dtype=np.float32).reshape(2, -1, 4)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    s32 = np.float32(float(sp))
    pos = np.zeros((nx * ny * nz, 4), np.float32)
    for a, idx in enumerate((i, j, k)):
        pos[:, a] = np.float32(2.5) + idx.ravel().astype(np.float32) * s32
    sim = pbd.Sim(params, len(pos))
    sim.add_particles(pos, np.zeros_like(pos))
    sim.step(frames)
    sim.sync()
    st = sim.state()
    sim.close()
    assert np.array_equal(got[0], st["x"]) and np.array_equal(got[1], st["v"])
