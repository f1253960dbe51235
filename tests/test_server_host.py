"""Host-side bookkeeping of the serving runtime (CPU; no server is created).

poll_fast() looks up each finished ticket's arrival time and model in arrays
indexed by ticket.  Over a long run the tickets issued grow without bound,
but those in flight do not; the arrays must follow the tickets in flight.
"""
import numpy as np

from mpx_gb300.server import MPCServer


def _bookkeeping(size=8):
    s = object.__new__(MPCServer)
    s._t_arr = np.zeros(size)
    s._t_mod = np.zeros(size, dtype=np.int8)
    s._t_base = 0
    s._arrival = {}
    return s


def test_arrival_arrays_follow_the_tickets_in_flight():
    rng = np.random.default_rng(0)
    s = _bookkeeping()
    truth = {}
    next_ticket = 0
    largest = 0
    for step in range(4000):
        # submit a burst (as submit / submit_many do: the tickets enter
        # _arrival before their arrival is noted)
        k = int(rng.integers(1, 40))
        tk = np.arange(next_ticket, next_ticket + k, dtype=np.int64)
        next_ticket += k
        times = rng.random(k) + step
        models = rng.integers(0, 2, k).astype(np.int8)
        for t, a, m in zip(tk.tolist(), times, models):
            s._arrival[t] = ("episode", 12, a)
            truth[t] = (a, m)
        s._note_arrival(tk, times, models)
        largest = max(largest, s._t_arr.shape[0])
        # finish a random subset of the outstanding tickets, in any order;
        # keep at most ~300 in flight
        out = np.array(sorted(s._arrival), dtype=np.int64)
        n_done = int(rng.integers(0, len(out) + 1)) if len(out) < 300 else len(out) - 150
        done = rng.choice(out, size=n_done, replace=False)
        t_arr, t_mod = s._arrivals(done)
        for t, a, m in zip(done.tolist(), t_arr, t_mod):
            assert (a, m) == truth.pop(t)
            del s._arrival[t]
    assert next_ticket > 50000
    # bounded by the tickets in flight (a few hundred), not the ~80k issued
    assert largest <= 4096, largest
    # every ticket still outstanding is still found
    out = np.array(sorted(s._arrival), dtype=np.int64)
    t_arr, t_mod = s._arrivals(out)
    for t, a, m in zip(out.tolist(), t_arr, t_mod):
        assert (a, m) == truth[t]


def test_a_burst_larger_than_the_arrays_grows_them():
    s = _bookkeeping(size=8)
    tk = np.arange(5, 105, dtype=np.int64)
    for t in tk.tolist():
        s._arrival[t] = None
    s._note_arrival(tk, tk * 0.5, (tk % 2).astype(np.int8))
    a, m = s._arrivals(tk)
    assert np.array_equal(a, tk * 0.5) and np.array_equal(m, tk % 2)
    assert s._t_arr.shape[0] >= 100

