"""Autotuner search and cache logic on the host, with a fake engine whose replay
time depends on the knob settings."""
import time

from ansatzevolve_gb300 import autotune as at
from ansatzevolve_gb300 import HAM_ON_THE_FLY, TUNE_CTAS_PER_SM, TUNE_OTF_THREADS, TUNE_PASS_OPS


class FakeEngine:
    def __init__(self, delay):
        self.delay = delay

    def launch_io(self):
        time.sleep(self.delay)

    def io_get_results(self):
        return None

    def close(self):
        pass


def test_greedy_search_finds_the_fastest_and_caches(tmp_path):
    # fastest at ctas 4, pass 5, threads 256
    cost = lambda t: 0.002 * (1 + abs(t[TUNE_CTAS_PER_SM] - 4) / 4 + abs(t[TUNE_PASS_OPS] - 5) +
                              abs(t[TUNE_OTF_THREADS] - 256) / 256)
    path = str(tmp_path / "tune.json")
    key = at.problem_key(10, 5, 5, 3, 192, HAM_ON_THE_FLY, True)
    assert key == "tups_N10_a5_b5_L3_nb192_otf_own"
    best, t, trials = at.tune(key, lambda tuning: FakeEngine(cost(tuning)), reps=2, path=path)
    assert best == {TUNE_CTAS_PER_SM: 4, TUNE_PASS_OPS: 5, TUNE_OTF_THREADS: 256, at.TUNE_SPMV_TPR: 0}
    # the default, then the other candidates of each knob: CTAs 3, pass size 2, threads 3
    assert len(trials) == 1 + 3 + 2 + 3
    assert at.lookup(key, path) == best
    assert at.lookup("other", path) == {}
