"""Host configuration surface: the flat ini reader (config.cpp:59-129,
config.h:122-159), per-group defaults and failure rules, derived constants
(kernel.cpp:25-41, properties.cpp:53-89, domain.cpp:37-49) and the .dat
readers (properties.cpp:7-33,91-116,164-189; host_data.cuh:24-115)."""
import numpy as np
import pytest

import sphnj_gb300 as S
from sphnj_gb300 import abi, cases

f32 = np.float32

MINIMAL = """
[time]
dt = 1e-4
iend = 10
[kernel]
smoothing_length = 0.012
particle_diameter = 0.01
[domain]
cell_xmin = -0.1
cell_xmax = 1.1
cell_ymin = -0.1
cell_ymax = 1.1
domain_xmin = 0
domain_xmax = 1
domain_ymin = 0
domain_ymax = 1
[solid]
auxetic_modulus = 2.0e8
"""


def read(tmp_path, text):
    f = tmp_path / "input.ini"
    f.write_text(text)
    return S.read_ini(f)


def test_defaults_and_keys(tmp_path):
    p, rc = read(tmp_path, MINIMAL)
    assert rc == abi.OK
    # defaults of the reference readParameter calls
    assert p.gravity[0] == 0.0 and p.gravity[1] == f32(-9.81)
    assert p.transient_type == abi.TRANSIENT
    assert p.particle_shift_coef == f32(0.4) and p.min_pressure == f32(-1.013e5)
    assert list(p.sound_speed) == [1500.0, 340.0]
    assert p.reference_density[1] == f32(1.29) and p.gamma[1] == f32(1.4)
    assert p.solid_reference_density == 2700.0 and p.youngs_modulus == f32(67.5e9)
    assert p.impact_length_hsml_ratio == 3.0 and p.thread_num == 32
    assert (p.solid_sub_step, p.result_interval, p.sort_every_step, p.shift_per_step) == (1, 1, 1, 1)
    # auxetic_modulus given, yield_strain 0 -> yield_strain = yield_stress / modulus
    assert p.yield_strain == f32(f32(2.0e7) / f32(2.0e8))


def test_comments_sections_overrides_and_bools(tmp_path):
    p, rc = read(tmp_path, MINIMAL + """
gravity = 1.0 ## direction is facing down
is_steady = NO
is_viscid = TRUE
is_plastic = n
is_2D_strain = 1
liquid_density = 5
liquid_density = 7   # the later one wins
""")
    assert rc == abi.OK
    assert p.gravity[1] == -1.0
    assert p.transient_type == abi.TRANSIENT
    assert p.is_fluid_viscid == 1
    assert p.plastic_type == abi.HYPER_ELASTIC
    assert p.constitution_type == abi.STRAIN_2D
    assert p.reference_density[0] == 7.0


@pytest.mark.parametrize("word,val", [("false", 0), ("F", 0), ("no", 0), ("N", 0), ("0", 0), ("none", 0),
                                      ("true", 1), ("yes", 1), ("-1", 1), ("anything", 1)])
def test_bool_words(tmp_path, word, val):
    p, _ = read(tmp_path, MINIMAL + f"is_viscid = {word}\n")
    assert p.is_fluid_viscid == val


def test_value_continuation_lines(tmp_path):
    # a line without '=' continues the previous value (config.cpp:87-116);
    # a value "false\n[fluid]" is not one of the false words -> true
    p, _ = read(tmp_path, MINIMAL + "is_viscid = false\n[fluid]\n")
    assert p.is_fluid_viscid == 1
    p, _ = read(tmp_path, MINIMAL + "is_viscid = false\n\n[fluid]\n")
    assert p.is_fluid_viscid == 0


def test_integer_keys_stop_at_exponent(tmp_path):
    p, _ = read(tmp_path, MINIMAL.replace("iend = 10", "iend = 1e5"))
    assert p.iend == 1  # "do not support 1e5 for integer" (cases/*/config/input.ini)


@pytest.mark.parametrize("old,new", [("dt = 1e-4", ""), ("smoothing_length = 0.012", ""),
                                     ("cell_xmax = 1.1", "cell_xmax = -0.1"),  # zero cell range
                                     ("domain_ymax = 1", "domain_ymax = 0"), ("auxetic_modulus = 2.0e8", ""),
                                     ("iend = 10", "iend = 0")])  # istart - iend == 0
def test_missing_required_keys_fail(tmp_path, old, new):
    p, rc = read(tmp_path, MINIMAL.replace(old, new))
    assert rc == abi.ERR_CONFIG


def test_one_sided_cell_range_is_accepted(tmp_path):
    # only a zero range fails (domain.cpp:22-26); a missing max defaults to 0
    p, rc = read(tmp_path, MINIMAL.replace("cell_xmax = 1.1", ""))
    assert rc == abi.OK and p.cell_xmax[0] == 0.0


def test_missing_file(tmp_path):
    with pytest.raises(S.SphnjError):
        S.read_ini(tmp_path / "nope.ini")


def test_derived_constants_match_reference_formulas(tmp_path):
    p, _ = read(tmp_path, MINIMAL + "liquid_sound_speed = 20\ngas_sound_speed = 20\nyoungs_modulus = 2e6\n"
                                    "poisson_ratio = 0.4\nsolid_density = 1000\n")
    p.fluid_number_total = 1
    S.derive(p)
    h, d, R = f32(0.012), f32(0.01), f32(3.0)
    assert p.smoothing_length_square == f32(h * h)
    assert p.smoothing_length_inverse == f32(f32(1) / h)
    assert p.impact_distance_square == f32(f32(R * R) * f32(h * h))
    assert p.kernel_coefficient_1 == np.exp(f32(-9.0), dtype=f32)
    hd = f32(h / d)
    hd3 = f32(np.power(np.float64(hd), -3.0))
    assert abs(p.kernel_coefficient_2 - f32(f32(f32(1) / f32(5.551921)) * hd3)) <= 1e-7 * p.kernel_coefficient_2
    kd = f32(f32(f32(2) / f32(5.551921)) * hd3) * f32(np.power(np.float64(h), -2.0))
    assert abs(p.kernel_differential - kd) <= 2e-7 * kd
    # cell grid, domain.cpp:37-49
    size = f32(R * h)
    n = int(f32(f32(1.1) - f32(-0.1)) / size)
    assert p.cell_number[0] == n and p.cell_number_total == n * p.cell_number[1]
    assert p.interval[0] == f32(f32(f32(1.1) - f32(-0.1)) / f32(n))
    assert p.interval_inv[0] == f32(f32(1) / p.interval[0])
    # EOS and solid constants, properties.cpp:53-89
    c2 = f32(np.power(np.float64(f32(20)), -2.0))
    assert abs(p.coefficient_p2rho[0] - f32(f32(7) * c2) / f32(1000)) <= 1e-7 * p.coefficient_p2rho[0]
    assert p.min_density[0] == f32(f32(0.6) * f32(1000))
    E, v = f32(2e6), f32(0.4)
    assert p.lambda_ == f32(f32(f32(E * v) / f32(1 - v)) / f32(1 + v))
    assert p.nu == f32(f32(E / f32(1 + v)) / f32(2))
    assert p.solid_sound_speed == f32(np.sqrt(f32(E / f32(f32(3) * f32(1 - f32(2) * v))) / f32(1000)))


def test_dat_round_trip_and_count_checks(tmp_path):
    case = cases.gate(dx=0.004, gas=True, layers=2)
    case.write(tmp_path / "c")
    p, arr = S.load_case(tmp_path / "c")
    assert (p.fluid_number[0], p.fluid_number[1], p.solid_number, p.virt_number) == \
           (case.n_liquid, case.n_gas, case.n_solid, case.n_virt)
    for k, a in case.arrays().items():
        assert np.array_equal(arr[k], a), k
    # header count != line count -> ERR_COUNT (properties.cpp:24-30)
    f = tmp_path / "c" / "data" / "virt_particle.dat"
    lines = f.read_text().splitlines()
    f.write_text("\n".join(lines[:-1]) + "\n")
    with pytest.raises(S.SphnjError) as e:
        S.load_case(tmp_path / "c")
    assert e.value.code == abi.ERR_COUNT


def test_solid_boundary_column_is_optional(tmp_path):
    case = cases.beam(dx=0.01)
    case.write(tmp_path / "b")
    f = tmp_path / "b" / "data" / "solid_particle.dat"
    rows = f.read_text().splitlines()
    # drop the boundary column as the reference's own generators do
    f.write_text("\n".join([rows[0]] + [" ".join(r.split()[:7]) for r in rows[1:]]) + "\n")
    p, arr = S.load_case(tmp_path / "b")
    assert np.all(arr["solid_boundary_type"] == 0)


# order of the derived parameters the reference-build harness dumps
# (oracle/ref/harness.cu `param_f` / `param_i`)
PARAM_F = ["smoothing_length_square", "smoothing_length_inverse_square", "impact_distance_square",
           "kernel_coefficient_1", "kernel_coefficient_2", "kernel_differential", "coefficient_3d_to_2d",
           ("interval", 0), ("interval", 1), ("interval_inv", 0), ("interval_inv", 1),
           ("coefficient_p2rho", 0), ("coefficient_p2rho", 1), ("coefficient_rho2p", 0),
           ("coefficient_rho2p", 1), ("gamma_inv", 0), ("gamma_inv", 1), ("min_density", 0), ("min_density", 1),
           "lambda_", "nu", "bulk_modulus", "solid_sound_speed", "dt", ("gravity", 1),
           ("reference_density_inverse", 0), ("reference_density_inverse", 1)]
PARAM_I = [("cell_number", 0), ("cell_number", 1), "cell_number_total", "fluid_number_total", "solid_number",
           "virt_number"]


def _field(p, f):
    return getattr(p, f[0])[f[1]] if isinstance(f, tuple) else getattr(p, f)


@pytest.mark.parametrize("name", ["water", "gas", "beam", "gate", "auxetic", "gate_air"])
def test_derived_parameters_equal_the_reference_builds(name):
    """The constants sphnj_params_derive gives (from the case's input.ini and
    particle counts, through the library's own ini reader) are bit-identical
    to the ones the reference's own build derived for the same case
    (Parameter::initiate: kernel.cpp:25-41, properties.cpp:53-89,
    domain.cpp:37-49), as its harness dumped them in the golden fixture."""
    from helpers import golden, golden_case

    if golden(name) is None:
        pytest.skip("fixture not generated")
    case, gz = golden_case(name)
    p = case.params()
    ref_f = np.asarray(gz["s0/param_f"], np.float32)
    ref_i = np.asarray(gz["s0/param_i"], np.int32)
    assert len(ref_f) == len(PARAM_F) and len(ref_i) == len(PARAM_I) + 1
    got_f = np.array([_field(p, f) for f in PARAM_F], np.float32)
    got_i = np.array([_field(p, f) for f in PARAM_I], np.int32)
    bad = [(PARAM_F[k], float(got_f[k]), float(ref_f[k])) for k in range(len(PARAM_F))
           if got_f[k].view(np.int32) != ref_f[k].view(np.int32)]
    assert not bad, f"{name}: derived constants differ from the reference build's: {bad}"
    assert np.array_equal(got_i, ref_i[:len(PARAM_I)]), (got_i, ref_i)


@pytest.mark.parametrize("name", ["water", "gas", "beam", "gate", "auxetic", "gate_air"])
def test_oracle_derives_the_same_parameters(name):
    """The oracle's own ini reading and derivation (used where the product
    library must not be loaded, e.g. the reference arm of the benchmark)
    gives the library's parameters bit for bit, so both sides of every
    comparison start from the reference build's constants."""
    import oracle
    from helpers import golden, golden_case

    if golden(name) is None:
        pytest.skip("fixture not generated")
    case, gz = golden_case(name)
    a, b = case.params(), oracle.params_for(case)
    differ = [f for f, _ in abi.Params._fields_ if bytes(a)[getattr(abi.Params, f).offset:][:getattr(abi.Params, f).size]
              != bytes(b)[getattr(abi.Params, f).offset:][:getattr(abi.Params, f).size]]
    assert not differ, f"{name}: the oracle's parameters differ from the library's in {differ}"
    ref_f = np.asarray(gz["s0/param_f"], np.float32)
    got_f = np.array([_field(b, f) for f in PARAM_F], np.float32)
    assert np.array_equal(got_f.view(np.int32), ref_f.view(np.int32))
