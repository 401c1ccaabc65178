"""Host logic of the set autotuner (databases_gpu_gb300/tune.py): size
classes, the set plan from per-class results, and the launch-cap choice,
fed made-up timings (no GPU)."""
import numpy as np

from databases_gpu_gb300 import tune


def test_size_class_is_floor_log2():
    assert [tune.size_class(x) for x in (1, 2, 3, 255, 256, 257, 1 << 20)] == [0, 1, 1, 7, 8, 8, 20]


def test_launch_cap_needs_a_clear_win_over_uncapped():
    def runner(times):
        return lambda cap: times[cap]
    assert tune.tune_launch(runner({0: 1.0, 2: 0.99, 4: 1.1, 8: 0.98})) == 0
    assert tune.tune_launch(runner({0: 1.0, 2: 0.99, 4: 1.1, 8: 0.96})) == 8
    assert tune.tune_launch(runner({0: 1.2, 2: 1.0, 4: 1.1, 8: 1.3})) == 2


def test_plan_takes_the_bucket_size_carrying_most_ops():
    r8 = tune.ClassResult(8, 100, {"bucket_bytes": 64, "num_subtables": 2, "max_evictions": 16},
                          50.0, {64: ({"bucket_bytes": 64, "num_subtables": 2,
                                       "max_evictions": 16}, 50.0),
                                 128: ({"bucket_bytes": 128, "num_subtables": 3,
                                        "max_evictions": 64}, 45.0)})
    r12 = tune.ClassResult(12, 5000, {"bucket_bytes": 128, "num_subtables": 4,
                                      "max_evictions": 256},
                           80.0, {64: ({"bucket_bytes": 64, "num_subtables": 3,
                                        "max_evictions": 64}, 70.0),
                                  128: ({"bucket_bytes": 128, "num_subtables": 4,
                                         "max_evictions": 256}, 80.0)})
    sizes = [300, 5000, 400]      # classes 8, 12, 8
    batches = [100, 5000, 120]    # class 12 carries most ops
    sb, d, ev = tune.plan_set(sizes, batches, {8: r8, 12: r12})
    assert sb == 128
    assert list(d) == [3, 4, 3] and list(ev) == [64, 256, 64]
    assert d.dtype == np.uint32 and ev.dtype == np.uint32
