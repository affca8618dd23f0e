"""Host logic of the checkpoint schedules, on the CPU: a mock trajectory whose
states are step indices checks that every reverse sweep visits each step once,
in reverse order and from the right state, and that the forward work it does
equals the plan's predicted cost."""
import pytest

from jaxfluids_gb300.adjoint import AdjointRK3


class Step(int):
    """A state that is its step index (cloned like a tensor)."""

    def clone(self):
        return self


class MockAdjoint(AdjointRK3):
    """States are integers (the step index); lam records the reversed steps."""

    def __init__(self):
        self.forward_steps = 0
        self.work = 0.0  # forward-step equivalents, stage recomputation included

    def advance(self, U, steps):
        self.forward_steps += steps
        self.work += steps
        return Step(U + steps)

    def step_vjp(self, U, lam):
        self.work += 2.0 / 3.0  # two stage states recomputed
        assert U == lam[-1] - 1, (U, lam)
        return lam + [U]

    def step_vjp_stages(self, U, U1, U2, lam):
        assert U == lam[-1] - 1 and U1 == ("s1", U) and U2 == ("s2", U)
        return lam + [U]

    def forward_stored(self, U0, nsteps):
        self.forward_steps += nsteps
        self.work += nsteps
        store = [(U0 + k, ("s1", U0 + k), ("s2", U0 + k)) for k in range(nsteps)]
        return Step(U0 + nsteps), store


@pytest.mark.parametrize("n,slots,leaf", [(1, 0, 1), (2, 0, 1), (12, 0, 1), (12, 2, 1), (12, 2, 4), (12, 0, 3),
                                          (37, 3, 1), (37, 3, 5), (200, 30, 1), (200, 4, 50), (200, 8, 40),
                                          (64, 1, 64), (50, 5, 7)])
def test_binomial_reverses_every_step_once(n, slots, leaf):
    a = MockAdjoint()
    UN, store, spine = a.forward_binomial(0, n, slots, leaf)
    assert UN == n
    assert a.forward_steps == n  # the loss's forward run places the first checkpoints
    a.work = 0.0
    lam = a.backward_binomial(store, spine, [n])
    assert lam == [n] + list(range(n - 1, -1, -1))
    assert a.work == pytest.approx(a.binomial_cost(n, slots, leaf))


def test_binomial_spine_holds_at_most_slots_states():
    a = MockAdjoint()
    for n, slots, leaf in ((200, 4, 50), (100, 6, 1), (37, 3, 5)):
        _, _, (parts, _) = a.forward_binomial(0, n, slots, leaf)
        # spine states plus the running one
        assert len([p for p in parts if p[2] > 0]) <= slots + 1


def test_leaf_memory_shortens_recomputation():
    a = MockAdjoint()
    plain = a.binomial_cost(200, 30, 1)
    leafy = a.binomial_cost(200, 4, 50)
    assert leafy < plain
    # with leaf memory for the whole run nothing is recomputed
    assert a.binomial_cost(40, 0, 40) == 0.0


@pytest.mark.parametrize("n,every", [(12, 12), (12, 4), (13, 5), (1, 3)])
def test_uniform_reverses_every_step_once(n, every):
    a = MockAdjoint()
    UN, ckpt = a.forward_uniform(Step(0), n, every)
    assert UN == n and sorted(ckpt) == list(range(0, n, every))
    for keep in (True, False):
        lam = a.backward_uniform(ckpt, n, every, [n], keep_stages=keep)
        assert lam == [n] + list(range(n - 1, -1, -1))


@pytest.mark.parametrize("n,every", [(12, 12), (12, 4), (13, 5), (1, 3), (1000, 50)])
def test_uniform_with_the_last_segment_kept_replays_all_but_it(n, every):
    for keep in (True, False):
        a = MockAdjoint()
        UN, ckpt = a.forward_uniform(Step(0), n, every, keep_last=True)
        assert UN == n and a.forward_steps == n and sorted(ckpt) == list(range(0, n, every))
        start = (n - 1) // every * every
        assert ckpt.last[0] == start and len(ckpt.last[1]) == n - start
        a.forward_steps = 0
        lam = a.backward_uniform(ckpt, n, every, [n], keep_stages=keep)
        assert lam == [n] + list(range(n - 1, -1, -1))
        # every segment but the kept one is replayed once (its last step too
        # when it keeps its stage states)
        replayed = start if keep else start - len([s for s in ckpt if s < start])
        assert a.forward_steps == replayed and ckpt.last is None
