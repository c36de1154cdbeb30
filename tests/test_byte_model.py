"""The byte model behind the reported roofline (sphnj_gb300/byte_model.py):
the per-pass tables add up to the closed step formula, the shifting pass's
per-launch figure averages its last pass in, and the mixed form's table
differs only where its fields do."""
from sphnj_gb300 import byte_model as bm

NF, NS, NV = 4_153_045, 0, 24_744


def test_plain_step_matches_the_closed_formula():
    for shifts in (0, 1, 2, 9, 10):
        for nf, ns, nv, k in ((NF, NS, NV, 1), (50_000, 3_000, 8_000, 4), (0, 5_200, 0, 1)):
            closed = (nf * (153 + 54 * shifts + 9 * (shifts > 0) + 16 * (shifts & 1)) if nf else 0) + nv * 46 + \
                ns * ((48 if nf else 20) + 440 * k)  # a solid's binning 20, its coupling 28 with fluid
            assert bm.step_bytes(nf, ns, nv, shifts, k) == closed, (shifts, nf, ns, nv, k)
            assert bm.bytes_per_step(nf, ns, nv, shifts, k) == bm.step_bytes(nf, ns, nv, shifts, k)


def test_shifting_launch_averages_the_last_pass():
    for mixed in (False, True):
        t = bm.PER_PARTICLE_MIXED if mixed else bm.PER_PARTICLE
        per_launch = bm.bytes_per_launch("shift_pass", NF, NS, NV, mixed, shifts=10)
        assert per_launch == NF * (t["shift_pass"] + t["shift_last"] / 10)
        # ten launches carry the step's shifting bytes
        assert abs(10 * per_launch - NF * (10 * t["shift_pass"] + t["shift_last"])) < 1.0


def test_mixed_table_differs_only_where_its_fields_do():
    changed = {k for k in bm.PER_PARTICLE if bm.PER_PARTICLE[k] != bm.PER_PARTICLE_MIXED[k]}
    assert changed == {"bin", "fluid_pair", "fluid_update", "shift_pass", "shift_last", "solid_deformation",
                       "solid_force", "solid_update"}
    # the deferred velocity correction: fewer bytes per pass, more in the last
    assert bm.PER_PARTICLE_MIXED["shift_pass"] < bm.PER_PARTICLE["shift_pass"]
    assert bm.PER_PARTICLE_MIXED["shift_last"] > bm.PER_PARTICLE["shift_last"]


def test_measured_traffic_scales_with_the_particle_count():
    for mixed in (False, True):
        a = bm.measured_traffic_per_launch("shift_pass", 1_000_000, mixed)
        b = bm.measured_traffic_per_launch("shift_pass", 2_000_000, mixed)
        assert b == 2 * a > 0
    assert bm.measured_traffic_per_launch("bin", NF) is None
