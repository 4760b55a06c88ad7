"""The step loop's observers on the GPU -- rescale_velocity! and the position
log of simulate! (src/Simulator.jl:119-144, 241-245) -- against the FP64
oracle (ref_md_run_observed).

Bars: positions and velocities within 1e-5 of the FP64 run over 60 steps
(FP32 forces; the same bar as the plain integrator), logged frames within
1e-5 of the oracle's frames.  Observer intervals that do not divide the
rebuild interval exercise the device-decided conditional nodes; the eager
path (nd_md_step_times) must reproduce the captured graphs bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 512
SIDE = 8.5
TOL = 1e-5


def _state(nd):
    return nd.synth.lj_system(0x4E440001, N, SIDE, 0.8)


def _params(nd):
    return nd.md_params(cutoff=2.5, skin=0.3, dt=1e-3, box_hi=(SIDE,) * 3, rebuild_every=10)


def _oracle_params(oracle):
    return oracle.md_params(cutoff=2.5, box_hi=(SIDE,) * 3, dt=1e-3)


@pytest.mark.parametrize("every", [10, 15, 5])
def test_thermostat_matches_oracle(nd, oracle, every):
    x, v, _ = _state(nd)
    eng = nd.MDEngine(_params(nd), x, v)
    eng.set_thermostat(0.6, 0.5, every)
    eng.run(60)
    xg, vg, _ = eng.get()
    eng.close()
    xr, vr, _, _ = oracle.md_run_observed(_oracle_params(oracle), x, v, steps=60,
                                          thermo=(0.6, 0.5, every))
    xp, vp, _ = oracle.md_run(_oracle_params(oracle), x, v, steps=60)
    print(f"every {every}: max|dx| {np.abs(xg - xr).max():.2e} max|dv| {np.abs(vg - vr).max():.2e}"
          f" (thermostat moved v by {np.abs(vr - vp).max():.2e})")
    assert np.abs(vr - vp).max() > 1e-2  # the thermostat acted
    assert np.abs(xg - xr).max() < TOL
    assert np.abs(vg - vr).max() < TOL


def test_thermostat_with_masses_and_charges(nd, oracle):
    # Ti weights |v_i| by m_i (rescale_velocity!, Simulator.jl:130); the
    # rescaled half-step velocity keeps the per-atom dt/2 F/m of the next kick
    x, v, q = nd.synth.lj_system(0x4E440001, N, SIDE, 0.8, charges=True)
    m = 1.0 + np.random.default_rng(3).random(N)
    p = nd.md_params(coulomb_k=1.0, cutoff=2.5, skin=0.3, dt=1e-3, box_hi=(SIDE,) * 3,
                     rebuild_every=10)
    eng = nd.MDEngine(p, x, v, q, m)
    eng.set_thermostat(0.8, 0.7, 10)
    eng.run(40)
    xg, vg, _ = eng.get()
    eng.close()
    pr = oracle.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(SIDE,) * 3, dt=1e-3)
    xr, vr, _, _ = oracle.md_run_observed(pr, x, v, q=q, m=m, steps=40, thermo=(0.8, 0.7, 10))
    assert np.abs(xg - xr).max() < TOL
    assert np.abs(vg - vr).max() < TOL


@pytest.mark.parametrize("every", [5, 15])
def test_position_log_matches_oracle(nd, oracle, every):
    x, v, _ = _state(nd)
    eng = nd.MDEngine(_params(nd), x, v)
    frames = 60 // every
    eng.set_log(every, frames)
    eng.run(60)
    assert eng.log_count() == frames
    log = eng.log_read(0, frames)
    eng.close()
    _, _, _, ref = oracle.md_run_observed(_oracle_params(oracle), x, v, steps=60,
                                          log_every=every)
    assert log.shape == ref.shape
    assert np.abs(log - ref).max() < TOL


def test_log_ring_keeps_the_last_frames(nd, oracle):
    x, v, _ = _state(nd)
    eng = nd.MDEngine(_params(nd), x, v)
    eng.set_log(5, 4)
    eng.run(60)  # 12 frames into a ring of 4
    assert eng.log_count() == 12
    last = eng.log_read(8, 4)
    with pytest.raises(nd.NDError):
        eng.log_read(7, 2)
    eng.close()
    _, _, _, ref = oracle.md_run_observed(_oracle_params(oracle), x, v, steps=60, log_every=5)
    assert np.abs(last - ref[8:12]).max() < TOL


def test_eager_path_reproduces_graphs(nd):
    # nd_md_step_times runs every step eagerly (host-decided rebuilds and
    # observers); the captured windows decide on the device: same bits
    x, v, _ = _state(nd)
    out = []
    for eager in (False, True):
        eng = nd.MDEngine(_params(nd), x, v)
        eng.set_thermostat(0.6, 0.5, 15)
        eng.set_log(7, 10)
        if eager:
            eng.step_times(60)
        else:
            eng.run(60)
        xg, vg, _ = eng.get()
        out.append((xg, vg, eng.log_read(0, eng.log_count())))
        eng.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])


def test_simulate_returns_poslog(nd, oracle):
    x, v, _ = _state(nd)
    sys_ = nd.GenericObjectCollection(position=x, velocity=v)
    spec = nd.SimSpec(duration=30, stepwidth=1e-3, vDamp=0.5)
    clct = nd.GenericRandomCollector(N, (0, 0, 0), (SIDE,) * 3, temperature=0.6)
    poslog = nd.simulate_(sys_, spec, clct, log_every=1)
    assert poslog.shape == (31, N, 3)
    assert np.array_equal(poslog[0], x)
    _, vr, _, ref = oracle.md_run_observed(_oracle_params(oracle), x, v, steps=30,
                                           thermo=(0.6, 0.5, 10), log_every=1)
    assert np.abs(poslog[1:] - ref).max() < TOL
    assert np.abs(sys_.velocity - vr).max() < TOL


def test_thermostat_rejected_for_ensembles(nd):
    e = nd.synth.ensemble(nd.synth.SEED_ENSEMBLE, nsys=4, nmin=256, nmax=512)
    table = nd.systems_table(e["n_atoms"], e["sigma"], e["epsilon"], e["box_lo"], e["box_hi"])
    ens = nd.Ensemble(nd.md_params(cutoff=2.5, skin=0.3, dt=1e-3, rebuild_every=10), table,
                      e["x"], e["v"])
    with pytest.raises(nd.NDError):
        ens.set_thermostat(0.6, 0.5, 10)
    ens.close()
