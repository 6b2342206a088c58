"""The standalone driver (python -m mumfim_gb300.batched_fiber_only) on the
Network_2_7 golden case: job file and network files written in the
reference's formats, two replicated RVEs, FP64. Its stress and stiffness
equal the oracle's bit for bit, and the stress matches the reference's
printed golden as the parity tests check it."""
import json

import numpy as np
import pytest

from conftest import network_2_7, voigt_to_mat

pytestmark = pytest.mark.gpu


def test_driver_matches_oracle(lib_path, oracle, golden_2_7, tmp_path, capsys):
    from mumfim_gb300 import SolutionStrategy
    from mumfim_gb300.batched_fiber_only import main
    from mumfim_gb300.network_io import format_network, format_params
    g = golden_2_7
    net = network_2_7(g)
    (tmp_path / "net.txt").write_text(format_network(net))
    (tmp_path / "net.txt.params").write_text(format_params(net))
    F = [float(x) for x in np.array(g["F"]).ravel()]
    job = ("- Case: golden\n  Problem Definition:\n    Mesh: net.txt\n"
           f"    Deformation Gradient: [{', '.join(repr(x) for x in F)}]\n"
           "  Solution Strategy:\n    Solver Type: Explicit\n"
           f"    Viscous Damping Factor: {g['visc_damp_coeff']!r}\n")
    (tmp_path / "job.yaml").write_text(job)
    out = tmp_path / "out.json"
    assert main([str(tmp_path / "job.yaml"), "2", "--json", str(out)]) == 0
    printed = capsys.readouterr().out
    assert "Took:" in printed and "Orientation Computation Took:" in printed
    res = json.loads(out.read_text())
    s = SolutionStrategy(visc_damp_coeff=g["visc_damp_coeff"], residual_tol=1e-6)
    orc = oracle.OracleBatch([net, net], [s, s])
    rc, sig, _ = orc.run(np.array(F).reshape(1, 3, 3).repeat(2, 0))
    rc, C = orc.material_stiffness()
    np.testing.assert_array_equal(res["sigma"], sig[0])
    np.testing.assert_array_equal(res["stiffness"], np.asarray(C[0]).ravel())
    assert res["status"] == 0
    J = np.linalg.det(np.array(F).reshape(3, 3))
    gold = np.array(g["outputs"]["explicit_cpu_out"]["stress"][0])
    assert np.abs(voigt_to_mat(np.array(res["sigma"]) * J) - gold).max() <= 1e-5 * np.abs(gold).max()
