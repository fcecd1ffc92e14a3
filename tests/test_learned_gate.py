"""Host logic of the learned Kepler start that needs no GPU: the gate on
the orbital-phase feature (log(|dt| sqrt(m/r^3)), column 3), fitted from
measured update counts and the network's price in update equivalents."""

import types

import numpy as np

from tupan_gb300.learned import LearnedStart, N_PARAM, IN, H


def _features(phase):
    X = np.zeros((len(phase), 4))
    X[:, 3] = phase
    return X


def test_parameter_count_matches_the_layer_sizes():
    # 4 -> 64 -> 64 -> 1 with biases
    assert N_PARAM == IN * H + H + H * H + H + H + 1 == 4545


def test_gate_where_the_network_pays_for_itself():
    phase = np.linspace(-8.0, 0.0, 801)
    plain = np.full(phase.size, 2.0)
    learned = np.full(phase.size, 2.0)
    # long steps (phase > -2) save one update with the network
    plain[phase > -2.0] = 3.0
    obj = types.SimpleNamespace()
    gate = LearnedStart.fit_gate(obj, _features(phase), plain, learned, 0.05)
    assert obj.gate == gate
    assert -2.02 < gate < -1.98


def test_gate_shuts_the_network_off_when_it_never_pays():
    phase = np.linspace(-8.0, 0.0, 101)
    iters = np.full(phase.size, 2.0)
    obj = types.SimpleNamespace()
    gate = LearnedStart.fit_gate(obj, _features(phase), iters, iters, 0.05)
    assert gate == float("inf")


def test_gate_weighs_savings_against_cost():
    # a saving of 0.04 updates does not pay a price of 0.05; 0.06 does
    phase = np.linspace(-4.0, 0.0, 401)
    plain = np.full(phase.size, 2.04)
    learned = np.full(phase.size, 2.0)
    obj = types.SimpleNamespace()
    assert LearnedStart.fit_gate(obj, _features(phase), plain, learned,
                                 0.05) == float("inf")
    plain[:] = 2.06
    gate = LearnedStart.fit_gate(obj, _features(phase), plain, learned, 0.05)
    assert gate < -3.99
