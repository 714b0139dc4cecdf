"""Batched launch: every instance equals its own sequential run bit for bit, in the chain and flat
forms and for every cluster / CTA shape of the persistent form, after autotuning, and when handles
are also stepped on their own (which makes the chain form capture its graphs again)."""
import numpy as np
import pytest

from conftest import bitwise_equal
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu


def instances(n=10, steps=60, seed=3):
    return S.batch_instances(n, size=(14, 40), steps=steps, pml=4, n_boxes=4, seed=seed)


def sequential(scs, steps):
    from fdtd_gb300 import solver
    out = []
    for sc in scs:
        with solver.Simulation.from_scenario(sc, probe_capacity=steps) as sim:
            sim.step(steps)
            sim.synchronize()
            out.append((sim.fields(), sim.read_probes(0, steps)))
    return out


def batched(scs, chunks, config=None, tune=False):
    from fdtd_gb300 import solver
    steps = sum(chunks)
    sims = [solver.Simulation.from_scenario(sc, probe_capacity=steps) for sc in scs]
    try:
        with solver.Batch(sims) as b:
            if config:
                b.set_config(*config)
            if tune:
                assert b.tune(3) > 0
            for c in chunks:
                b.step(c)
            b.synchronize()
        assert all(s.current_step == steps for s in sims)
        return [(s.fields(), s.read_probes(0, steps)) for s in sims]
    finally:
        for s in sims:
            s.close()


def same(a, b):
    return all(bitwise_equal(x[0], y[0]) and bitwise_equal(x[1], y[1]) for x, y in zip(a, b))


@pytest.mark.parametrize("config", [(-1, 256), (0, 256), (1, 256), (2, 128), (4, 256), (8, 512)])
def test_batch_equals_sequential(gpu_lib, config):
    scs = instances()
    assert same(batched(scs, [25, 35], config), sequential(scs, 60))


def test_batch_after_tuning(gpu_lib):
    scs = instances(7, 40, seed=8)
    assert same(batched(scs, [40], tune=True), sequential(scs, 40))


@pytest.mark.parametrize("config", [None, (-1, 256)])
def test_handles_stepped_alone_between_launches(gpu_lib, config):
    from fdtd_gb300 import solver
    scs = instances(5, 40, seed=11)
    ref = sequential(scs, 40)
    sims = [solver.Simulation.from_scenario(sc, probe_capacity=40) for sc in scs]
    try:
        with solver.Batch(sims) as b:
            if config:
                b.set_config(*config)
            b.step(10)
            b.synchronize()
            sims[2].step(7)        # one instance moves on its own
            sims[2].synchronize()
            b.step(23)
            b.synchronize()
        for s in sims:
            if s.current_step < 40:
                s.step(40 - s.current_step)
        got = []
        for s in sims:
            s.synchronize()
            got.append((s.fields(), s.read_probes(0, 40)))
        assert [s.current_step for s in sims] == [40] * 5
        assert same(got, ref)
    finally:
        for s in sims:
            s.close()
