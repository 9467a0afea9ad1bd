"""Host logic of the warm-start evaluation on the CPU: the time to each
residual level from the residual histories of a plain and a warm-started
run, and the fallback to the identity grid when a warm grid folds."""
import pytest

from glemur_gb300 import train_warmstart as tw

# (seconds, attempts, residual, min Delta) every check
PLAIN = [(0.0, 0, 0.52, 1.0), (2.0, 200, 0.41, 0.9), (4.0, 400, 0.35, 0.9), (9.0, 900, 0.29, 0.9)]
WARM = [(0.1, 0, 0.85, 0.5), (1.0, 200, 0.38, 0.5), (2.0, 400, 0.28, 0.5), (3.0, 600, 0.24, 0.5)]


def test_first_reach():
    assert tw.first_reach(PLAIN, 0.4) == (4.0, 400)
    assert tw.first_reach(PLAIN, 0.41) == (2.0, 200)
    assert tw.first_reach(WARM, 0.3, offset=0.5) == (2.5, 400)
    assert tw.first_reach(PLAIN, 0.1) == (None, None)


def test_level_times_with_the_warm_cost_included():
    lv = tw.level_times(PLAIN, WARM, t_net=0.5, folded=False, levels=(0.4, 0.3, 0.25, 0.1))
    assert lv["0.4"] == dict(plain_s=4.0, plain_attempts=400, warm_s=1.5, warm_attempts=200,
                             speedup=pytest.approx(4.0 / 1.5))
    assert lv["0.3"]["plain_s"] == 9.0 and lv["0.3"]["warm_s"] == 2.5
    # reached only from the warm start: no speedup figure
    assert lv["0.25"]["plain_s"] is None and lv["0.25"]["warm_s"] == 3.5 and lv["0.25"]["speedup"] is None
    assert lv["0.1"] == dict(plain_s=None, plain_attempts=None, warm_s=None, warm_attempts=None, speedup=None)


def test_level_times_after_a_fold_fall_back_to_the_plain_run():
    folded = [(0.2, 0, 0.81, 0.4), (0.3, 22, 0.80, -29.0)]
    lv = tw.level_times(PLAIN, folded, t_net=1.5, folded=True, levels=(0.4, 0.3))
    # the plain run's times and attempts, plus the folded run's 1.8 s and 22 attempts
    assert lv["0.4"]["warm_s"] == pytest.approx(4.0 + 1.8) and lv["0.4"]["warm_attempts"] == 422
    assert lv["0.3"]["warm_s"] == pytest.approx(9.0 + 1.8)
    assert lv["0.4"]["speedup"] == pytest.approx(4.0 / 5.8)
