"""The streaming trainer's rolling pool (bartels_gb300.lpcg.train_stream), on
the CPU with a stand-in system generator and network: every pack's plan is
closed exactly once, after its last system has left the pool, no training
step uses a closed plan, and the counts of systems and steps are the ones
asked for."""
import numpy as np


def test_stream_pool_releases_each_plan_once_and_never_trains_on_a_closed_one():
    from bartels_gb300 import lpcg

    closed = []

    class FakePlan:
        def __init__(self, k):
            self.k = k
            self.handle = object()

        def close(self):
            assert self.handle is not None, "closed twice"
            closed.append(self.k)
            self.handle = None

    def fake_systems(ctx, count, seed, n_range=(8, 40), newton_iters=4, dt=0.01):
        plan = FakePlan(seed)
        for it in range(newton_iters):
            yield lpcg.System(plan, None, None, dict(instances=count, seed=seed, newton_iteration=it))

    class FakeNet:
        def __init__(self):
            self.used = []

        def train_step(self, plan, values, residual, **kw):
            assert plan.handle is not None, "trained on a closed plan"
            self.used.append(plan.k)
            return 0.25

    orig = lpcg.packed_newton_systems
    lpcg.packed_newton_systems = fake_systems
    try:
        net = FakeNet()
        hist, produced = lpcg.train_stream(net, None, systems=18, steps=12, per_pack=2, newton_iters=3, pool=4,
                                           seed=1)
    finally:
        lpcg.packed_newton_systems = orig
    seeds = [1 * 100003 + k for k in range(3)]  # three packs of 2 instances x 3 Newton systems
    assert produced == 18
    assert len(hist) == 12 and np.allclose(hist, 0.25)
    assert sorted(closed) == sorted(seeds)
    # the pool mixes packs: some step after the first pack's arrival trains on an older pack
    assert len(set(net.used)) == 3
