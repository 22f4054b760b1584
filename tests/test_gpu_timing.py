"""Phase timers (rt_tic / rt_toc / rt_timing_secs): the GPU counterpart of
the reference's tic/toc counters (timing_module.f90:34-75)."""
import pytest

from harness import configs
from raytracer_3d_gb300._lib import RtError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def test_phase_timers_measure_device_time():
    m = configs.build_model(configs.packet_small(), "fp64")
    try:
        with m.timed("main loop"):
            for _ in range(3):
                with m.timed("integrate"):
                    m.integrate(2)
                with m.timed("diag"):
                    m.diagnose(fields=False)
        t_int, n_int = m.timing_secs("integrate")
        t_diag, n_diag = m.timing_secs("diag")
        t_all, n_all = m.timing_secs("main loop")
        assert (n_int, n_diag, n_all) == (3, 3, 1)
        assert t_int > 0 and t_diag > 0
        assert t_all >= t_int + t_diag * 0.5          # the loop encloses both phases
        assert m.timing_secs("never started") == (0.0, 0)
        # reading resolves the events; later pairs add on
        with m.timed("integrate"):
            m.integrate(1)
        t2, n2 = m.timing_secs("integrate")
        assert n2 == 4 and t2 > t_int
        assert "integrate" in m.timing_summary()
    finally:
        m.close()


def test_timer_call_order_errors():
    m = configs.build_model(configs.shear_mini(), "fp64")
    try:
        with pytest.raises(RtError):
            m.toc("integrate")                        # toc before tic
        m.tic("integrate")
        with pytest.raises(RtError):
            m.tic("integrate")                        # running already
        m.toc("integrate")
    finally:
        m.close()
