"""Batched ensemble: one persistent launch per step over members of
different sizes gives each member exactly the result it gets alone."""
import numpy as np
import pytest

from harness import configs, interior

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def _members(count, seed, steps=7, spatial=(4, 6, 8), spectral=(4, 6, 8)):
    rng = np.random.default_rng(seed)
    return [configs.ensemble_member(rng, steps=steps, spatial=spatial, spectral=spectral) for _ in range(count)]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("tuning", [(8, 256, 0, 16), (3, 128, 1, 2), (1, 512, 0, 4), (4, 1024, 1, 6)])
def test_batch_equals_members_alone(precision, tuning):
    from raytracer_3d_gb300.batch import Batch
    exps = _members(6, seed=11)
    alone = []
    for e in exps:
        m = configs.build_model(e, precision)
        m.integrate(e.steps)
        alone.append(m.get_state().copy())
        m.close()
    models = [configs.build_model(e, precision) for e in exps]
    b = Batch(models)
    b.set_tuning(*tuning)
    b.integrate(3)
    b.integrate(4)          # 7 steps: graphs and single launches, both parities
    for e, m, ref in zip(exps, models, alone):
        got = m.get_state()
        sl = interior(e.n)
        assert np.array_equal(got[sl], ref[sl]), e.n
    # one launch per step per member class present (at most three)
    assert b.launch_count() in (7, 14, 21)
    b.close()
    for m in models:
        m.close()


def test_member_can_leave_and_step_alone():
    from raytracer_3d_gb300.batch import Batch
    exps = _members(3, seed=5)
    ref = []
    for e in exps:
        m = configs.build_model(e, "fp32")
        m.integrate(5)
        ref.append(m.get_state().copy())
        m.close()
    models = [configs.build_model(e, "fp32") for e in exps]
    b = Batch(models)
    b.integrate(2)
    models[1].integrate(1)   # one member steps on its own stream between batch calls
    b2 = Batch([models[0], models[2]])
    b2.integrate(3)
    models[1].integrate(2)
    for e, m, r in zip(exps, models, ref):
        sl = interior(e.n)
        assert np.array_equal(m.get_state()[sl], r[sl])
    b.close()
    b2.close()
    for m in models:
        m.close()


@pytest.mark.parametrize("persistent", [256, 512, 128, 0])
def test_mixed_classes_equal_members_alone(persistent):
    """members whose planes fill the warp-specialised CTA take that kernel,
    small planes its z-slice form, the rest the group / plane kernels, in
    one captured step; every member gets its result alone"""
    from raytracer_3d_gb300.batch import Batch
    rng = np.random.default_rng(23)
    exps = [configs.ensemble_member(rng, steps=5, spatial=(8, 16, 24, 32), spectral=(4, 6)) for _ in range(7)]
    exps.append(configs.ensemble_member(np.random.default_rng(3), steps=5, spatial=(32,), spectral=(4,)))
    exps.append(configs.ensemble_member(np.random.default_rng(4), steps=5, spatial=(6,), spectral=(4,)))
    alone = []
    for e in exps:
        m = configs.build_model(e, "fp32")
        m.integrate(e.steps)
        alone.append(m.get_state().copy())
        m.close()
    models = [configs.build_model(e, "fp32") for e in exps]
    b = Batch(models)
    b.set_tuning(4, 256, 0, 2)
    b.set_persistent(persistent)
    npers = b.persistent_members()
    if persistent:
        assert 0 < npers < len(exps)      # the 32x32 member qualifies, the 6x6x6 one never
    else:
        assert npers == 0
    b.integrate(2)
    b.integrate(3)          # graphs and a single launch, both parities
    for e, m, ref in zip(exps, models, alone):
        sl = interior(e.n)
        assert np.array_equal(m.get_state()[sl], ref[sl]), e.n
    # one launch per class present: warp-specialised planes, z slices, group / plane
    assert b.launch_count() in ((5, 10, 15) if persistent else (5,))
    b.close()
    for m in models:
        m.close()


@pytest.mark.parametrize("threads", [256, 512])
def test_fused_launch_equals_two_launches_and_alone(threads):
    """members of both warp-specialised classes (planes that fill the CTA,
    small planes in z slices) stepped by ONE launch per step give each
    member exactly its result alone, as the two launches per step do"""
    from raytracer_3d_gb300.batch import Batch
    dims = [(32, 16, 4, 4, 2, 4), (32, 32, 4, 2, 2, 4), (8, 8, 8, 4, 4, 2), (8, 8, 8, 2, 4, 4), (16, 8, 4, 2, 2, 2)]
    exps = [configs.shear_mini(n=n, seed=40 + i) for i, n in enumerate(dims)]
    alone = []
    for e in exps:
        m = configs.build_model(e, "fp32")
        m.integrate(5)
        alone.append(m.get_state().copy())
        m.close()
    for fused in (True, False):
        models = [configs.build_model(e, "fp32") for e in exps]
        b = Batch(models)
        b.set_tuning(4, 256, 0, 2)
        b.set_persistent(threads)
        b.set_fused(fused)
        assert b.persistent_members() == len(exps)
        l0 = b.launch_count()
        b.integrate(2)
        b.integrate(3)          # graphs and a single launch, both parities
        assert b.launch_count() - l0 == (5 if fused else 10), fused
        for e, m, ref in zip(exps, models, alone):
            sl = interior(e.n)
            assert np.array_equal(m.get_state()[sl], ref[sl]), (fused, e.n)
        b.close()
        for m in models:
            m.close()
