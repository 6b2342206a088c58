"""Job-file reader (the fiber_only.yaml format) on CPU."""
import numpy as np
import pytest

JOB = """# two cases in the reference's job-file layout
- Case: Shear test
  Problem Definition:
    Mesh: nets/net_a.txt
    #Deformation Gradient: [9, 9]
    Deformation Gradient: [1.01, 0.002, -.003, 0, 1, 0, 0, 0, .99]
  Solution Strategy:
    Solver Type: Explicit
    Convergence Tolerance: 1E-6
    Load Time: 10
    Amplitude Type: Smooth Step
    Viscous Damping Factor: 50 # per unit mass
    Critical Time Scale Factor: 0.5
    Detect Oscillation:
      Type: Iteration Only
      Max Iterations: 200
  Output:
    3D Orientation Tensor: true
    2D Orientation Tensor: [ true, [0,0,1]]
- Case: "second"
  Problem Definition:
    Mesh: b.txt
    Deformation Gradient: [1,0,0,0,1,0,0,0,1]
  Solution Strategy:
    Solver Type: Explicit
    Viscous Damping Factor: 1
"""


def test_reads_cases(tmp_path):
    from mumfim_gb300.jobfile import load_micro_cases
    p = tmp_path / "job.yaml"
    p.write_text(JOB)
    cases = load_micro_cases(str(p))
    assert [c.name for c in cases] == ["Shear test", "second"]
    a = cases[0]
    assert a.mesh == "nets/net_a.txt"
    np.testing.assert_array_equal(a.F, [1.01, 0.002, -0.003, 0, 1, 0, 0, 0, 0.99])
    assert a.solution["Detect Oscillation"]["Max Iterations"] == 200
    assert a.solution["Convergence Tolerance"] == 1e-6
    assert a.orientation_2d_axis == [0.0, 0.0, 1.0]
    s = a.strategy()
    assert s.visc_damp_coeff == 50.0 and s.crit_time_scale_factor == 0.8
    assert cases[1].orientation_2d_axis is None


@pytest.mark.parametrize("bad, msg", [
    (JOB.replace("Solver Type: Explicit\n    Convergence", "Solver Type: Implicit\n    Convergence"),
     "Explicit"),
    (JOB.replace("[1.01, 0.002, -.003, 0, 1, 0, 0, 0, .99]", "[1, 0, 0]"), "9 entries"),
    (JOB.replace("    Mesh: b.txt\n", ""), "missing field"),
    (JOB.replace("[ true, [0,0,1]]", "[ true, [0,0,1]"), "flow sequence"),
    ("Case: x\n", "sequence of cases"),
])
def test_rejects_bad_jobs(tmp_path, bad, msg):
    from mumfim_gb300.jobfile import JobFileError, load_micro_cases
    p = tmp_path / "job.yaml"
    p.write_text(bad)
    with pytest.raises(JobFileError, match=msg):
        load_micro_cases(str(p))
