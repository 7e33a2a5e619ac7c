"""A horizon that continues a finished run (kura_set_horizon after kura_run).

The reference resumes an integration through fs.dat and -R (kuramoto.cu:466-494, 543): the
phases, t and h are read back and the output grid is rebuilt from int(t/dt)+1.  The library
continues on the device instead, keeping the phases, the FSAL slope and the step size, so a run
cut into horizons takes exactly the steps of one uninterrupted run: same accepted steps, the
same records at every output time both runs emit, bitwise the same final phases.
"""
import numpy as np
import pytest

from helpers import normal_inputs

pytestmark = pytest.mark.gpu
DENSE, VOLCANO = 0, 1
PERSISTENT, TENSOR = 1, 2


def _net(native, n, coupling, engine, thetas, om, cs):
    B = len(thetas)
    net = native.Network(n, k=5, coupling=coupling, batch=B, seed=3, dense_level=0, engine=engine)
    net.set_frequencies(om)
    if coupling == DENSE:
        net.generate_adjacency()
    for b in range(B):
        net.set_coupling(b, cs[b])
        net.set_state(b, thetas[b], 0.0, 0.005)
    return net


def _records(net, B, store):
    def on_out(b, idx, te, r, th, cp):
        store[b].append((round(te, 9), r))
    net.run(on_output=on_out)


@pytest.mark.parametrize("coupling,engine,batch", [(VOLCANO, PERSISTENT, 3), (DENSE, PERSISTENT, 2),
                                                   (DENSE, TENSOR, 16)])
def test_continued_horizons_equal_one_run(native, coupling, engine, batch):
    n = 700
    _, om = normal_inputs(n, 5)
    thetas = [normal_inputs(n, 40 + b, init=2 * np.pi)[0] for b in range(batch)]
    cs = [1.0 + 0.5 * (b % 7) for b in range(batch)]
    dt, ends = 0.5, (2.0, 4.0, 6.0)

    one = _net(native, n, coupling, engine, thetas, om, cs)
    one.set_horizon(ends[-1], dt, True)
    rec1 = {b: [] for b in range(batch)}
    _records(one, batch, rec1)
    st1 = one.stats()
    fin1 = [one.state(b) for b in range(batch)]
    one.close()

    cut = _net(native, n, coupling, engine, thetas, om, cs)
    rec2 = {b: [] for b in range(batch)}
    for i, t1 in enumerate(ends):
        cut.set_horizon(t1, dt, i == 0)
        _records(cut, batch, rec2)
    st2 = cut.stats()
    fin2 = [cut.state(b) for b in range(batch)]
    cut.close()

    assert st1["accepted"] == st2["accepted"] and st1["rejected"] == st2["rejected"]
    for b in range(batch):
        assert fin1[b][1] == fin2[b][1] and fin1[b][2] == fin2[b][2]  # t and h
        assert np.array_equal(fin1[b][0], fin2[b][0])
        d1 = dict(rec1[b])
        assert len(rec1[b]) == int(ends[-1] / dt) + 1
        # a record between a horizon's end and the overshoot of its last step is not emitted
        # (the resumed grid starts after the trajectory's time, as the reference's does)
        assert len(rec2[b]) >= len(rec1[b]) - len(ends) + 1
        for te, r in rec2[b]:
            assert d1[te] == r, (b, te)


def test_horizon_needs_fresh_or_finished_trajectories(native):
    n = 200
    _, om = normal_inputs(n, 6)
    th = normal_inputs(n, 7)[0]
    net = _net(native, n, VOLCANO, PERSISTENT, [th, th], om, [1.0, 2.0])
    net.set_horizon(1.0, 0.5, True)
    net.run()
    net.set_state(0, th, 0.0, 0.005)  # trajectory 0 fresh, trajectory 1 finished
    with pytest.raises(native.KuraError):
        net.set_horizon(2.0, 0.5, False)
    net.set_state(1, th, 0.0, 0.005)
    net.set_horizon(2.0, 0.5, False)
    net.run()
    net.close()


@pytest.mark.parametrize("coupling,engine,batch,chunk", [(VOLCANO, PERSISTENT, 3, 5), (DENSE, TENSOR, 16, 4)])
def test_advance_in_chunks_equals_one_run(native, coupling, engine, batch, chunk):
    """kura_advance: a run cut into budgets of step attempts takes the steps of one run and
    delivers the same records, with every trajectory active until it reaches the end."""
    n = 600
    _, om = normal_inputs(n, 9)
    thetas = [normal_inputs(n, 60 + b, init=2 * np.pi)[0] for b in range(batch)]
    cs = [1.5 + 0.5 * (b % 5) for b in range(batch)]

    one = _net(native, n, coupling, engine, thetas, om, cs)
    one.set_horizon(5.0, 0.25, True)
    rec1 = {b: [] for b in range(batch)}
    _records(one, batch, rec1)
    st1 = one.stats()
    fin1 = [one.state(b) for b in range(batch)]
    one.close()

    cut = _net(native, n, coupling, engine, thetas, om, cs)
    cut.set_horizon(5.0, 0.25, True)
    rec2 = {b: [] for b in range(batch)}
    calls, running = 0, batch
    while running:
        running = cut.advance(chunk, on_output=lambda b, i, te, r, th, cp: rec2[b].append((round(te, 9), r)) and False)
        calls += 1
        assert calls < 10000
    st2 = cut.stats()
    fin2 = [cut.state(b) for b in range(batch)]
    cut.close()

    assert calls > 3
    assert st1["accepted"] == st2["accepted"] and st1["rejected"] == st2["rejected"]
    for b in range(batch):
        assert rec1[b] == rec2[b], b
        assert fin1[b][1] == fin2[b][1] and np.array_equal(fin1[b][0], fin2[b][0])


def test_resume_through_host_state_on_the_tensor_engine(native):
    """The pattern of a -R resume per budget: read every trajectory's phases, t and h to the
    host, set them back (each with its own t and h), set the horizon and advance again.  The
    Cauchy frequencies give oscillators with |omega| in the hundreds, so the phases grow large
    and the trajectories' times spread apart."""
    from helpers import cauchy_inputs
    n, batch = 2000, 16
    _, om = cauchy_inputs(n, 5)
    thetas = [cauchy_inputs(n, 70 + b)[0] for b in range(batch)]
    net = _net(native, n, DENSE, TENSOR, thetas, om, [3.0] * batch)
    net.set_horizon(20.0, 0.01, True)
    for _ in range(6):
        net.advance(64)
    for _ in range(8):
        st = [net.state(b) for b in range(batch)]
        assert len({round(s[1], 12) for s in st}) > 1
        for b in range(batch):
            net.set_state(b, st[b][0], st[b][1], st[b][2])
        net.set_horizon(20.0, 0.01, False)
        net.advance(64)
        for b in range(batch):
            r = net.order(b)
            assert r.size > 0 and np.all(np.isfinite(r)) and np.all((r >= 0) & (r <= 1.0 + 1e-6))
    net.close()
