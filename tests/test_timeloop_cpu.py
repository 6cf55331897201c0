"""The reference main loop's step sequence (phd_gb300.izem.TimeLoop, izem.f90:252-281)
on a recording stand-in for the device context: the order of the calls,
the half steps, the time carried, and the FIXEDDT branch of timestep
(module_solver.f90:240-244)."""
import types

import numpy as np

from phd_gb300.izem import CHEM_BDF, TimeLoop


class Recorder:
    def __init__(self, dt=2e-3, dtmax=5.0):
        self.calls = []
        self.adi = types.SimpleNamespace(time_ref=1e-7)
        self._dt, self._dtmax = dt, dtmax

    def timestep(self, DTmax, dtmin):
        self.calls.append(("timestep", DTmax, dtmin))
        return np.full(4, self._dt), self._dt

    def reaction_selec(self, dt, mode, time):
        self.calls.append(("chem", dt, mode, time))
        return self._dtmax

    def rk3(self, dt, time0):
        self.calls.append(("rk3", dt, time0))


def test_strang_sequence_and_carried_state():
    r = Recorder()
    loop = TimeLoop(r, reaction=True, chem_mode=CHEM_BDF, time=1.0)
    loop.step()
    loop.step()
    kinds = [c[0] for c in r.calls]
    assert kinds == ["timestep", "chem", "rk3", "chem"] * 2
    # the second time step sees the first step's dtmin and the chemistry's DTmax
    assert r.calls[4][1:] == (5.0, 2e-3)
    # half steps, the stage time of rk3, the time of the second half step
    assert r.calls[1][1] == 1e-3 and r.calls[1][3] == 1.0
    assert r.calls[2] == ("rk3", 2e-3, 1.0)
    assert r.calls[3][3] == 1.0 + 2e-3
    assert loop.time == 1.0 + 4e-3


def test_fixed_time_step_skips_the_criteria():
    r = Recorder()
    loop = TimeLoop(r, reaction=True, fixed_dt=3e-9)
    dt = loop.step()
    assert dt == 3e-9 / 1e-7
    assert "timestep" not in [c[0] for c in r.calls]
    assert np.all(loop.dt4 == dt)
    assert r.calls[0] == ("chem", 0.5 * dt, CHEM_BDF, 0.0)


def test_without_chemistry_only_rk3():
    r = Recorder()
    loop = TimeLoop(r, reaction=False)
    loop.step(dt=1e-3)
    assert [c[0] for c in r.calls] == ["timestep", "rk3"]
    assert r.calls[1] == ("rk3", 1e-3, 0.0)
