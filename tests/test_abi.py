"""CPU tests of the C ABI boundary: the library loads, exports every function include/pbd.h
declares, and the host-only entry points (defaults, config grammar, range checks) behave
like the reference's Config/Communication code.  No GPU: nothing here launches a kernel."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "pbd.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pbd_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(pbd):
    L = pbd.lib()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(pbd.EXPORTED)


def test_abi_version_and_struct_size(pbd):
    assert pbd.lib().pbd_abi_version() == 1
    p = pbd.default_params()
    assert p.struct_size == C.sizeof(pbd.Params) == 128


def test_defaults_are_config_txt(pbd):
    p = pbd.default_params()
    assert p.threads_per_block == 512
    assert p.particle_radius == pytest.approx(0.5)
    assert p.max_neighbours_per_particle == 512
    assert p.delta_t == pytest.approx(0.01)
    assert p.gravity == pytest.approx(-29.82)
    assert p.rest_density == 1200
    assert p.kernel_width_spiky == pytest.approx(6.1)
    assert p.k_scorr == pytest.approx(0.2) and p.n_scorr == 4 and p.q_scorr == pytest.approx(0.2)
    assert p.c_viscosity == pytest.approx(1e-4) and p.kernel_width_poly == pytest.approx(4.1)
    assert p.e_vorticity == 1.0
    assert p.collision_type == 0 and p.kernel_width_neighbours == 2 and p.max_collision_batches == 16
    assert p.stiffness == pytest.approx(0.3)
    assert list(p.bounds_min) == [1.5] * 3 and list(p.bounds_max) == [62.5] * 3
    assert p.solver_iterations == 1 and p.stabilization_iterations == 1
    assert p.active == pbd.ACTIVE_ALL
    assert p.max_grid == 128 ** 3
    assert p.lambda_epsilon == pytest.approx(1e-4)
    assert p.flags == pbd.FLAG_CELL_END_QUIRK
    assert pbd.lib().pbd_validate_params(C.byref(p)) == 0


CONFIG = """
// a config in the reference's grammar
#define ON 1
Application:
{
  Cuda: { threadsPerBlock = 256; }
  name = "a \\"string\\" with ; and : inside";   /* block comment
     spanning lines */
  Simulation:
  {
    Active:
    {
      applyForces = ON;
      computeVorticity = false;
      computeViscosity = 0;
    }
    Density:
    {
      restDensity = 950;
      kernelWidthSpiky = 1.5;
      nSCorr = 3;
    }
    Enclosure:
    {
      enclosurePositionDamping = 0.25f;
      X: { min = 2.0; max = 30.5; }
    }
    Iterations: { solverIterations = 4; }
    Forces:
    {
      gravity = -9.82;   // comment after a value
      deltaT = 0.0166667;
    }
  }
}
"""


def test_parse_config_grammar(pbd):
    p = pbd.parse_config(CONFIG)
    assert p.threads_per_block == 256
    assert p.active & pbd.ACTIVE["applyForces"]
    assert not p.active & pbd.ACTIVE["computeVorticity"]
    assert not p.active & pbd.ACTIVE["computeViscosity"]
    assert p.active & pbd.ACTIVE["computeLambda"]          # untouched key keeps its default
    assert p.rest_density == 950 and p.kernel_width_spiky == 1.5 and p.n_scorr == 3
    assert p.enclosure_position_damping == 0.25
    assert p.bounds_min[0] == 2.0 and p.bounds_max[0] == 30.5 and p.bounds_max[1] == 62.5
    assert p.solver_iterations == 4
    assert p.gravity == pytest.approx(-9.82) and p.delta_t == pytest.approx(0.0166667)


def test_config_include_and_roundtrip(pbd, tmp_path):
    inc = tmp_path / "inc.txt"
    inc.write_text("Application: { Simulation: { Collision: { stiffness = 0.75; } } }\n")
    main = tmp_path / "main.txt"
    main.write_text('#include "inc.txt"\nApplication: { Simulation: { Forces: { gravity = 3.5; } } }\n')
    p = pbd.load_config(str(main))
    assert p.stiffness == 0.75 and p.gravity == 3.5
    out = tmp_path / "written.txt"
    assert pbd.lib().pbd_write_config(C.byref(p), os.fsencode(str(out))) == 0
    q = pbd.load_config(str(out), pbd.default_params())
    for f, _ in pbd.Params._fields_:
        a, b = getattr(p, f), getattr(q, f)
        if isinstance(a, float):
            assert a == pytest.approx(b, rel=1e-6), f
        elif isinstance(a, int):
            assert a == b, f
    assert list(p.bounds_min) == list(q.bounds_min)
    text = out.read_text()
    assert "Application:\n{\n" in text and "  Simulation:\n" in text


def test_config_errors(pbd, tmp_path):
    with pytest.raises(pbd.PBDError) as e:
        pbd.load_config(str(tmp_path / "missing.txt"))
    assert e.value.code == pbd.ERR_CONFIG
    with pytest.raises(pbd.PBDError) as e:
        pbd.parse_config("Application: { Forces: { gravity = ; } }")
    assert e.value.code == pbd.ERR_CONFIG
    with pytest.raises(pbd.PBDError):
        pbd.parse_config("Application: { Forces: { gravity = 1; }")   # unclosed scope


@pytest.mark.parametrize("field,value", [
    ("gravity", 1000.5), ("kernel_width_neighbours", 0), ("kernel_width_neighbours", 51), ("c_viscosity", -0.1),
    ("e_vorticity", 1e5), ("rest_density", 0.0), ("rest_density", 1e6), ("kernel_width_spiky", 0.0),
    ("kernel_width_poly", 1001.0), ("solver_iterations", 101), ("stabilization_iterations", 101), ("delta_t", 0.0),
    ("delta_t", 11.0), ("collision_type", 2), ("max_collision_batches", 0), ("max_collision_batches", 513),
    ("stiffness", 1.5), ("k_scorr", -101.0), ("n_scorr", 101), ("q_scorr", 100.5),
    ("enclosure_position_damping", 1.1), ("enclosure_velocity_damping", -0.1),
])
def test_setter_ranges(pbd, field, value):
    # Communication.h:440-624
    p = pbd.default_params()
    setattr(p, field, value)
    assert pbd.lib().pbd_validate_params(C.byref(p)) == pbd.ERR_RANGE
    assert b"out of range" in pbd.lib().pbd_last_error()


def test_enclosure_ranges(pbd):
    p = pbd.default_params()
    p.bounds_min[1] = 1.0
    assert pbd.lib().pbd_validate_params(C.byref(p)) == pbd.ERR_RANGE
    p = pbd.default_params()
    p.bounds_max[2] = 127.0
    assert pbd.lib().pbd_validate_params(C.byref(p)) == pbd.ERR_RANGE
    p = pbd.default_params()
    p.bounds_min[0], p.bounds_max[0] = 10.0, 10.0
    assert pbd.lib().pbd_validate_params(C.byref(p)) == pbd.ERR_RANGE


def test_null_arguments(pbd):
    L = pbd.lib()
    assert L.pbd_params_default(None) == pbd.ERR_INVALID_ARG
    assert L.pbd_step(None, 1, None) == pbd.ERR_INVALID_ARG
    assert L.pbd_destroy(None) == pbd.OK
    p = pbd.default_params()
    assert L.pbd_create(C.byref(p), 16, None) == pbd.ERR_INVALID_ARG


def test_cpp_host_example_links_and_parses_its_arguments(pbd):
    """The C++ host example (examples/dam_break.cpp) is built against libpbd.so alone; without
    arguments it prints its usage before touching the GPU."""
    import subprocess
    exe = os.path.join(ROOT, "pbd-simulation-framework-cuda_gb300", "examples", "dam_break")
    if not os.path.exists(exe):
        import build as pkg_build
        pkg_build.build_examples(force=True)
    r = subprocess.run([exe, "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
