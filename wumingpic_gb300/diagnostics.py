"""Energy history and Weibel growth-rate diagnostics.

The reference records the energy history (2d/proj/weibel/app.f90:479-545: time,
particle kinetic energy, electric and magnetic field energy, total) and
leaves the growth-rate analysis to the user.  ``growth_rate`` fits the linear
phase of the magnetic energy: a least-squares line through ln E_B over the
rising branch between ``lo`` and ``hi`` times the first maximum.
"""
import numpy as np


def energy_history(run_step, energy, nsteps, every, dt):
    """Advance ``nsteps`` steps in chunks of ``every``; return (t, E) with E[:, k] =
    [kinetic(species...), E field, B field] as the reference's energy_history sums."""
    t, rows = [0.0], [np.array(energy())]
    done = 0
    while done < nsteps:
        k = min(every, nsteps - done)
        run_step(k)
        done += k
        t.append(done * dt)
        rows.append(np.array(energy()))
    return np.array(t), np.array(rows)


def growth_rate(t, eb, lo=1e-3, hi=0.1):
    """Exponential growth rate of the field amplitude (half the rate of E_B) in the
    linear phase: ln E_B fitted on the rising branch where lo*E_max <= E_B <= hi*E_max,
    E_max being the first maximum.  Returns (gamma, (t0, t1), npoints)."""
    t = np.asarray(t, float)
    eb = np.asarray(eb, float)
    imax = int(np.argmax(eb))
    emax = eb[imax]
    rise = np.arange(imax + 1)
    sel = rise[(eb[rise] >= lo * emax) & (eb[rise] <= hi * emax)]
    if len(sel) < 3:
        raise ValueError("linear phase not resolved")
    # the contiguous last run of selected points before the maximum
    breaks = np.nonzero(np.diff(sel) > 1)[0]
    if len(breaks):
        sel = sel[breaks[-1] + 1:]
    slope, _ = np.polyfit(t[sel], np.log(eb[sel]), 1)
    return 0.5 * slope, (float(t[sel[0]]), float(t[sel[-1]])), len(sel)
