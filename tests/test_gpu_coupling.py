"""Macro/micro record exchange through the C ABI (mfg_batch_micro_fo_*)
against the oracle: each micro_fo_result holds the FP64 stress and stiffness
bit for bit (zeros in the averaged-volume-stress slots), each
micro_fo_step_result the two orientation tensors (1e-14, as the orientation
tests), over two successive macro iterations."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_micro_fo_iterations_match_oracle(lib_path, oracle):
    from mumfim_gb300 import coupling as CP
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=3, n_nodes=700, steps=400)
    params = np.zeros((3, CP.NUM_PARAM_FIELDS))
    params[:, CP.FIBER_RADIUS] = [1e-3, 2e-3, 5e-4]
    params[:, CP.VOLUME_FRACTION] = [0.1, 0.2, 0.05]
    params[:, CP.ORIENTATION_AXIS_X:CP.ORIENTATION_AXIS_Z + 1] = [[0, 0, 1.0], [1.0, 0, 0],
                                                                  [0.3, 0.4, 0.5]]
    with CP.MicroFOBatch(w.networks, params, w.strategies, precision="f64") as mb:
        for net, prm in zip(w.networks, params):
            assert net.scale_factor == oracle.scale_conversion(
                net.coords, net.connectivity, prm[CP.FIBER_RADIUS], prm[CP.VOLUME_FRACTION])
        orc = oracle.OracleBatch(w.networks, w.strategies)
        step = mb.step_results()
        np.testing.assert_allclose(step[:, :9], orc.orientation_3d().reshape(3, 9), rtol=0,
                                   atol=1e-14)
        F2 = np.repeat((np.eye(3) + 0.01 * np.array([[0, 1.0, 0], [0, 0, 0], [0, 0, -1]]))[None],
                       3, 0)
        for F in (w.F, F2):
            res = mb.iterate(F.reshape(3, 9))
            rc, sig, _ = orc.run(F)
            rc, Co = orc.material_stiffness()
            np.testing.assert_array_equal(res[:, :6], sig)
            assert (res[:, 6:9] == 0).all()
            np.testing.assert_array_equal(res[:, 9:], np.asarray(Co).reshape(3, 36))
            assert (mb.last_status["status"] == 0).all()
            step = mb.step_results()
            np.testing.assert_allclose(step[:, :9], orc.orientation_3d().reshape(3, 9), rtol=0,
                                       atol=1e-14)
            normal = params[:, CP.ORIENTATION_AXIS_X:CP.ORIENTATION_AXIS_Z + 1]
            np.testing.assert_allclose(step[:, 9:], orc.orientation_2d(normal).reshape(3, 9),
                                       rtol=0, atol=1e-14)
