"""The serving loop's adaptive kernel shape (csrc/serve_policy.h), on the CPU:
the arrival-rate estimate and the shape each launch takes, driven by
simulated Poisson arrivals of requests log-uniform in 1..2048 items (the
serving benchmark's mix) and a dispatcher that looks every millisecond."""
import ctypes

import numpy as np
import pytest

STEP = 0.001  # s between dispatcher looks
LOW, HIGH = 0, 1
SWITCH = 15.0e6  # items/s


@pytest.fixture(scope="module")
def hc():
    from _paths import build_hostcheck

    lib = ctypes.CDLL(build_hostcheck())
    lib.hc_shape_policy_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    return lib


def arrivals(segments, seed=1):
    """Items accepted per step: segments of (seconds, items/s) of Poisson
    request arrivals with log-uniform sizes; returns the cumulative count."""
    rng = np.random.default_rng(seed)
    mean = np.mean(np.floor(np.exp(rng.uniform(0, np.log(2048), 400000))))
    per_step = []
    for seconds, items_per_s in segments:
        n = int(round(seconds / STEP))
        reqs = rng.poisson(items_per_s / mean * STEP, size=n)
        sizes = np.floor(np.exp(rng.uniform(0, np.log(2048), int(reqs.sum())))).astype(np.int64)
        idx = np.repeat(np.arange(n), reqs)
        per_step.append(np.bincount(idx, weights=sizes, minlength=n).astype(np.int64))
    return np.cumsum(np.concatenate(per_step)).astype(np.uint64)


def run(hc, items_cum, switch=SWITCH, fixed=LOW):
    n = len(items_cum)
    shapes = np.zeros(n, np.int32)
    rates = np.zeros(n, np.float64)
    hc.hc_shape_policy_run(LOW, HIGH, switch, fixed, items_cum.ctypes.data, n, STEP, shapes.ctypes.data, rates.ctypes.data)
    return shapes, rates


def test_below_the_switch_rate_keeps_the_low_shape(hc):
    # 85% of the switch rate (the benchmark's half-load level sits there) for 60 s
    shapes, rates = run(hc, arrivals([(60.0, 0.85 * SWITCH)]))
    assert (shapes == LOW).all()
    steady = rates[5000:]
    assert abs(steady.mean() / (0.85 * SWITCH) - 1) < 0.02  # unbiased
    assert steady.std() / steady.mean() < 0.05  # about 3% scatter


def test_a_step_above_switches_within_tens_of_ms(hc):
    shapes, _ = run(hc, arrivals([(0.5, 0.0), (1.0, 1.5 * SWITCH)]))
    start = 500
    assert (shapes[:start] == LOW).all()
    first_high = start + int(np.argmax(shapes[start:] == HIGH))
    assert shapes[first_high] == HIGH and first_high - start <= 60  # ms
    assert (shapes[first_high:] == HIGH).all()  # and stays there


def test_hysteresis_and_the_way_back(hc):
    # high load, then 90% of the switch rate (between the thresholds), then none
    shapes, _ = run(hc, arrivals([(1.0, 1.5 * SWITCH), (5.0, 0.9 * SWITCH), (1.0, 0.0)]))
    assert (shapes[500:1000] == HIGH).all()
    assert (shapes[1000:6000] == HIGH).all()  # 90%: keeps the running shape
    back = 6000 + int(np.argmax(shapes[6000:] == LOW))
    assert shapes[back] == LOW and back - 6000 <= 150  # ms
    assert (shapes[back:] == LOW).all()


def test_from_high_below_80_percent_returns(hc):
    shapes, _ = run(hc, arrivals([(1.0, 1.5 * SWITCH), (5.0, 0.7 * SWITCH)]))
    assert shapes[999] == HIGH
    assert (shapes[1300:] == LOW).all()


def test_fixed_shape_without_a_switch_rate(hc):
    shapes, _ = run(hc, arrivals([(1.0, 3.0 * SWITCH)]), switch=0.0, fixed=2)
    assert (shapes == 2).all()
