"""The output schedule of the time averages (dsmcField timeProperties,
dsmcField.C:113-150, with controlDict's writeInterval): at every output time
the averages of the window just ended stay readable, and they restart before
the next step while resetAtOutput is on; resets stop after the first output
time t with t + deltaT > resetAtOutputUntilTime."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CORNER = os.path.join(HERE, "golden", "cases", "hypersonic_corner")
COUETTE = os.path.join(HERE, "golden", "cases", "couette_N2-O2")
PLATE = os.path.join(HERE, "golden", "cases", "supersonic_flat_plate")


def test_schedule_is_read_from_the_case(gpu_lib):
    from hystrath_gb300.dsmc import parse_case
    s = parse_case(CORNER)           # runTime, writeInterval 1e-4 s, deltaT 1e-6 s
    assert s.write_interval_steps == 100 and s.reset_at_output == 1
    assert s.reset_at_output_until_time == 1.5e-3
    c = parse_case(COUETTE)          # adjustableRunTime, writeInterval 1 s, deltaT 1e-5 s
    assert c.write_interval_steps == 100_000 and c.reset_at_output_until_time == 0.5
    p = parse_case(PLATE)
    assert p.write_interval_steps == 100 and p.reset_at_output_until_time == 8e-3
    assert s.measure_errors == 0 and s.measure_heat_flux_shear_stress == 0


@pytest.mark.gpu
def test_schedule_restarts_the_averages_like_a_manual_reset(gpu_lib):
    """The corner case stepped 1800 steps with its schedule equals the same
    case without a schedule and one reset after step 1500 (the last reset
    output), field for field; at an output time the window just ended is
    still readable."""
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    s = parse_case(CORNER)
    a = DsmcCloud(s)
    a.initialise()
    a.evolve(300)
    assert a.info().sample_steps == 100      # the window 200..300, not yet restarted
    a.evolve(1)
    assert a.info().sample_steps == 1        # restarted before step 301
    a.evolve(1499)
    s2 = parse_case(CORNER)
    s2.reset_at_output = 0
    b = DsmcCloud(s2)
    b.initialise()
    b.evolve(1500)
    b.reset_sampling()
    b.evolve(300)
    assert a.info().sample_steps == b.info().sample_steps == 300
    for f in ("rhoN", "Ttra", "Ux", "p"):
        np.testing.assert_array_equal(a.field(f), b.field(f), err_msg=f)
    a.close()
    b.close()
