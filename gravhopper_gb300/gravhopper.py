"""Host API mirroring ``gravhopper.gravhopper``: ``Simulation``, ``IC`` and the exceptions.

The names, arguments, defaults and state layout follow gravhopper/gravhopper.py:68-1785:
``Simulation(dt, eps, algorithm='tree')``, ``add_IC``, ``run(N)``, ``reset``, ``snap``,
``current_snap``, ``prev_snap``, ``perform_timestep``, ``calculate_acceleration``,
``add_external_force`` (and the time- and velocity-dependent variants),
``positions``/``velocities`` of shape (Nsnap, Np, 3), ``masses`` (Np), ``times`` (Nsnap).

What differs is where the work runs: ``run`` keeps the particles on the GPU and
executes every drift-kick-drift step (gravhopper.py:405-416) there, one fused launch
per step, writing each step's state into device history buffers that are copied to
the host once per call.  When external forces are registered, each step falls back to
the host for those callbacks (they are arbitrary Python), with the N-body force still
computed on the GPU.

Extensions: ``theta`` (opening angle, default 0.7 as gravhopper/jbgrav.py:52) and
``precision`` ('fp64' default; 'mixed' for the direct sum).

Units: with astropy importable, Quantities in and out as in the reference; otherwise
plain numbers in kpc, km/s, Msun, Myr.
"""
from __future__ import annotations

import time

import numpy as np

from . import ics as _ics
from . import jbgrav
from . import units as U

# Snapshot history per device run segment (positions and velocities, 48 bytes per
# particle and step); one segment's copy to the host overlaps the next one's steps.
HISTORY_SEGMENT_BYTES = 256 << 20


class GravHopperException(Exception):
    """Base of the errors this module raises (the reference's class names, so that
    callers' except clauses keep working)."""


class UninitializedSimulationException(GravHopperException):
    """run() or a snapshot accessor was called before any particles were added."""


class ICException(GravHopperException):
    """Initial conditions are malformed (a key missing, lengths that disagree, an IC
    generator called without its parameters); the message is also printed, as the
    reference does."""

    def __init__(self, msg):
        super().__init__(msg)
        print(msg)


class UnknownAlgorithmException(GravHopperException):
    """The force algorithm is neither 'tree' nor 'direct'."""


class ExternalPackageException(GravHopperException):
    """A feature that needs galpy, gala, agama or pynbody was called; those packages
    are not part of this engine.  The message is also printed."""

    def __init__(self, msg):
        super().__init__(msg)
        print(msg)


class DeviceForce(object):
    """An external force evaluated on the GPU: ``fn`` takes CUDA float64 tensors
    (positions in kpc, velocities in km/s; time as a float in Myr) and returns the
    acceleration in km/s/Myr as a tensor of shape (N,3) or one that broadcasts to it.
    Simulation.run calls it on the device-resident state, with no host copies.  Called
    with host arrays (Simulation.calculate_acceleration), it moves them to the current
    CUDA device and returns a numpy array.  No counterpart in the reference, whose
    external forces are host functions (gravhopper.py:603-845)."""

    def __init__(self, fn):
        if not callable(fn):
            raise ExternalPackageException("A device force must be callable.")
        self.fn = fn

    def __call__(self, pos, *rest):
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())

        def to_dev(a, unit):
            return torch.as_tensor(np.ascontiguousarray(U.value(a, unit), dtype=np.float64), device=dev)
        args = list(rest)
        if len(args) == 2:  # (time, args): a scalar; (vel, args): an (N,3) array
            args[0] = float(U.value(args[0], U.TIME)) if np.ndim(args[0]) == 0 else to_dev(args[0], U.VELOCITY)
        out = self.fn(to_dev(pos, U.LENGTH), *args)
        return U.quantity(torch.as_tensor(out).cpu().numpy(), U.ACCEL)


def _default(q_astropy, plain):
    return q_astropy() if U.HAVE_ASTROPY else plain


class Simulation(object):
    """Main class for an N-body simulation (gravhopper/gravhopper.py:91-163)."""

    def __init__(self, dt=None, eps=None, algorithm="tree", theta=0.7, precision="fp64"):
        if dt is None:
            dt = _default(lambda: 1 * U._u.Myr, 1.0)
        if eps is None:
            eps = _default(lambda: 100 * U._u.pc, 0.1)
        self.ICarrays = False
        self.Np = 0
        self.Nsnap = 0
        self.timestep = 0
        self.running = False
        self._pos = None   # (Nsnap, Np, 3) kpc
        self._vel = None   # (Nsnap, Np, 3) km/s
        self._mass = None  # (Np) Msun
        self._times = None  # (Nsnap) Myr
        self.extra_force_functions = []
        self.extra_timedependent_force_functions = []
        self.extra_velocitydependent_force_functions = []
        self.lenunit, self.velunit, self.massunit, self.timeunit = U.LENGTH, U.VELOCITY, U.MASS, U.TIME
        self.accelunit = U.ACCEL
        self.params = {}
        self.set_dt(dt)
        self.set_eps(eps)
        self.set_algorithm(algorithm)
        self.set_theta(theta)
        self.set_precision(precision)

    # ---- parameters (gravhopper.py:166-290) ----------------------------------
    def set_dt(self, dt):
        """Sets the simulation time step (time dimensions; plain numbers are Myr)."""
        U.value(dt, U.TIME, "dt")
        self.params["dt"] = dt

    def get_dt(self):
        return self.params["dt"]

    def set_eps(self, eps):
        """Sets the gravitational softening length (plain numbers are kpc)."""
        U.value(eps, U.LENGTH, "eps")
        self.params["eps"] = eps

    def get_eps(self):
        return self.params["eps"]

    def set_algorithm(self, algorithm):
        """'tree' (Barnes-Hut) or 'direct' (direct summation)."""
        if algorithm in ("tree", "direct"):
            self.params["algorithm"] = algorithm
        else:
            raise ValueError("algorithm must be 'tree' or 'direct'.")

    def get_algorithm(self):
        return self.params["algorithm"]

    def set_theta(self, theta):
        """Opening angle of the tree walk in radians (default 0.7)."""
        theta = float(theta)
        if not theta >= 0.0:
            raise ValueError("theta must be >= 0.")
        self.params["theta"] = theta

    def get_theta(self):
        return self.params["theta"]

    def set_precision(self, precision):
        """'fp64' (reference arithmetic) or 'mixed' (FP32 pair arithmetic with compensated
        sums; for the tree, the accepted cells' interactions, with the same opening
        decisions).  State and integration stay FP64 either way."""
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'.")
        self.params["precision"] = precision

    def get_precision(self):
        return self.params["precision"]

    def _dt(self):
        return float(U.value(self.params["dt"], U.TIME, "dt"))

    def _eps(self):
        return float(U.value(self.params["eps"], U.LENGTH, "eps"))

    # ---- state arrays ------------------------------------------------------------
    @property
    def positions(self):
        return None if self._pos is None else U.quantity(self._pos, U.LENGTH)

    @property
    def velocities(self):
        return None if self._vel is None else U.quantity(self._vel, U.VELOCITY)

    @property
    def masses(self):
        return None if self._mass is None else U.quantity(self._mass, U.MASS)

    @property
    def times(self):
        return None if self._times is None else U.quantity(self._times, U.TIME)

    # ---- running (gravhopper.py:293-342) ---------------------------------------
    def run(self, N=1):
        """Run N timesteps; initialises on the first call, continues afterwards.
        Afterwards run_stats() describes this call (steps, wall time, throughput)."""
        N = int(N)
        t_start = time.perf_counter()
        host = self._has_extra_forces()
        self._run(N)
        self._record_run(N, time.perf_counter() - t_start, host)

    def _run(self, N):
        if not self.running:
            self.init_run(N)
        else:
            self.Nsnap += N
            self._pos = np.concatenate((self._pos, np.zeros((N, self.Np, 3))), axis=0)
            self._vel = np.concatenate((self._vel, np.zeros((N, self.Np, 3))), axis=0)
            self._times = np.concatenate((self._times, np.zeros(N)), axis=0)
        if self._has_extra_forces():
            self._run_device_external(N)
            return
        self._run_device(N)

    def _record_run(self, N, seconds, host):
        np_ = int(self.Np)
        pairs = np_ * (np_ - 1) if self.params["algorithm"] == "direct" else None
        self._last_run = {"steps": max(N, 0), "particles": np_, "seconds": seconds,
                          "algorithm": self.params["algorithm"], "precision": self.params["precision"],
                          "path": "device, external forces" if host else "device",
                          "particle_steps_per_s": np_ * max(N, 0) / seconds if seconds > 0 else None,
                          "pairs_per_s": (pairs * max(N, 0) / seconds if pairs is not None and seconds > 0
                                          else None)}

    def run_stats(self):
        """Statistics of the last run() call: steps, particles, wall-clock seconds
        (history copies included), particle steps per second and, for the direct sum,
        pair interactions per second; algorithm, precision and whether external forces
        were evaluated each step.  None before any run."""
        return None if getattr(self, "_last_run", None) is None else dict(self._last_run)

    def _has_extra_forces(self):
        return bool(self.extra_force_functions or self.extra_timedependent_force_functions
                    or self.extra_velocitydependent_force_functions)

    def _run_device(self, N):
        import torch

        from . import engine
        if N <= 0:
            return
        t0 = self.timestep
        dev = torch.device("cuda", torch.cuda.current_device())
        x = torch.from_numpy(np.ascontiguousarray(self._pos[t0])).to(dev)
        v = torch.from_numpy(np.ascontiguousarray(self._vel[t0])).to(dev)
        m = torch.from_numpy(np.ascontiguousarray(self._mass)).to(dev)
        # Segments of about 256 MB of snapshot history: segment k is copied into the
        # history arrays by a helper thread on a side stream while segment k + 1 runs
        # (the copies into pageable host memory return only when complete).
        seg = max(1, min(N, HISTORY_SEGMENT_BYTES // max(1, 48 * self.Np)))
        pending, pool, copy_stream = None, None, None
        done = 0
        try:
            while done < N:
                k = min(seg, N - done)
                hp, hv = engine.run_dkd(x, v, m, k, self._dt(), self._eps(), algorithm=self.params["algorithm"],
                                        precision=self.params["precision"], theta=self.params["theta"],
                                        hist_stride=1)
                if k == N:  # one segment: copy straight into the history arrays
                    torch.from_numpy(self._pos[t0 + 1:t0 + N + 1]).copy_(hp)
                    torch.from_numpy(self._vel[t0 + 1:t0 + N + 1]).copy_(hv)
                    break
                if pool is None:
                    from concurrent.futures import ThreadPoolExecutor
                    pool = ThreadPoolExecutor(max_workers=1)
                    copy_stream = torch.cuda.Stream(device=dev)
                ready = torch.cuda.Event()
                ready.record(torch.cuda.current_stream(dev))
                if pending is not None:
                    pending.result()
                pending = pool.submit(self._copy_history, hp, hv, ready, copy_stream, t0 + done + 1)
                done += k
            if pending is not None:
                pending.result()
        finally:
            if pool is not None:
                pool.shutdown(wait=True)
        dt = self._dt()
        for k in range(t0 + 1, t0 + N + 1):
            self._times[k] = self._times[k - 1] + dt
        self.timestep = t0 + N

    def _force_fn(self):
        from . import engine
        p = self.params
        if p["algorithm"] == "direct":
            return lambda x, m, out: engine.direct_force(x, m, self._eps(), precision=p["precision"], out=out)
        if p["algorithm"] == "tree":
            return lambda x, m, out: engine.tree_force(x, m, self._eps(), p["theta"], precision=p["precision"],
                                                       out=out)
        raise UnknownAlgorithmException()

    def _run_device_external(self, N):
        """Steps with external forces, state resident on the device: per step the first
        drift, the N-body force and the external accelerations (device forces on the
        device; host functions on a copy of the half-drifted positions, their result
        copied back), then the kick and second drift, and the snapshot copied into the
        history.  The same arithmetic and order as perform_timestep with
        calculate_acceleration (gravhopper.py:405-473)."""
        import torch

        from . import engine
        if N <= 0:
            return
        force = self._force_fn()
        dev = torch.device("cuda", torch.cuda.current_device())
        t0 = self.timestep
        dt = self._dt()
        x = torch.from_numpy(np.ascontiguousarray(self._pos[t0])).to(dev)
        v = torch.from_numpy(np.ascontiguousarray(self._vel[t0])).to(dev)
        m = torch.from_numpy(np.ascontiguousarray(self._mass)).to(dev)
        xh = torch.empty_like(x)
        acc = torch.empty_like(x) if self.Np > 1 else None
        ext = torch.empty_like(x)
        host = [fn for fns in self._external_lists() for fn, _ in fns if not isinstance(fn, DeviceForce)]
        xh_host = torch.empty((self.Np, 3), dtype=torch.float64, pin_memory=True) if host else None
        for k in range(N):
            t = t0 + k + 1
            engine.dkd_drift(x, v, dt, out=xh)
            if acc is not None:
                force(xh, m, acc)
            self._external_on_device(xh, v, ext, xh_host, t)
            engine.dkd_kick_drift(xh, v, acc, ext, dt, out=x)
            torch.from_numpy(self._pos[t]).copy_(x)
            torch.from_numpy(self._vel[t]).copy_(v)
            self._times[t] = self._times[t - 1] + dt
            self.timestep = t

    def _external_lists(self):
        return (self.extra_force_functions, self.extra_timedependent_force_functions,
                self.extra_velocitydependent_force_functions)

    def _external_on_device(self, xh, v, ext, xh_host, t):
        """ext = 0 + each registered force in the reference's order (gravhopper.py:462-473),
        at the half-drifted positions xh, time t_(t-1) + dt/2 and the step's starting
        velocities."""
        import torch
        kick_time = self._times[t - 1] + 0.5 * self._dt()
        ext.zero_()
        pos_host = None
        for kind, fns in zip(("pos", "time", "vel"), self._external_lists()):
            for fn, args in fns:
                if isinstance(fn, DeviceForce):
                    extra = (xh,) if kind == "pos" else (xh, kick_time) if kind == "time" else (xh, v)
                    r = fn.fn(*extra, args)
                    if not isinstance(r, torch.Tensor) or r.device != ext.device:
                        raise ExternalPackageException("A device force must return a tensor on the state's device.")
                    ext.add_(r.to(torch.float64))
                    continue
                if pos_host is None:
                    xh_host.copy_(xh)
                    pos_host = U.quantity(xh_host.numpy(), U.LENGTH)
                if kind == "pos":
                    r = fn(pos_host, args)
                elif kind == "time":
                    r = fn(pos_host, U.quantity(kick_time, U.TIME), args)
                else:
                    r = fn(pos_host, U.quantity(self._vel[t - 1], U.VELOCITY), args)
                r = np.asarray(U.value(r, U.ACCEL, "acceleration"), dtype=np.float64)
                ext.add_(torch.from_numpy(np.ascontiguousarray(r)).to(ext.device))

    def _copy_history(self, hp, hv, ready, stream, first):
        import torch
        with torch.cuda.stream(stream):
            stream.wait_event(ready)
            k = hp.shape[0]
            torch.from_numpy(self._pos[first:first + k]).copy_(hp)
            torch.from_numpy(self._vel[first:first + k]).copy_(hv)

    def init_run(self, Nsnap=None):
        """Allocates the (Nsnap, Np, 3) position and velocity histories and puts the ICs in
        slot 0 (gravhopper.py:324-342)."""
        if self.ICarrays is False:
            raise UninitializedSimulationException
        self.Nsnap = Nsnap + 1
        self.Np = len(self.ICarrays["pos"])
        self._pos = np.zeros((self.Nsnap, self.Np, 3))
        self._vel = np.zeros((self.Nsnap, self.Np, 3))
        self._mass = np.zeros(self.Np)
        self._times = np.zeros(self.Nsnap)
        self._pos[0] = U.value(self.ICarrays["pos"], U.LENGTH, "pos")
        self._vel[0] = U.value(self.ICarrays["vel"], U.VELOCITY, "vel")
        self._mass[:] = U.value(self.ICarrays["mass"], U.MASS, "mass")
        self.running = True

    def reset(self):
        """Drops the run's histories and times; the ICs and registered external forces stay."""
        self.running = False
        self._pos = self._vel = self._mass = self._times = None
        self.Nsnap = 0
        self.timestep = 0

    def snap(self, step):
        """dict with 'pos' (Np,3), 'vel' (Np,3), 'mass' (Np) of snapshot ``step``."""
        return {"pos": U.quantity(self._pos[step], U.LENGTH), "vel": U.quantity(self._vel[step], U.VELOCITY),
                "mass": U.quantity(self._mass, U.MASS)}

    def current_snap(self):
        return self.snap(self.timestep)

    def prev_snap(self):
        return self.snap(self.timestep - 1)

    def perform_timestep(self):
        """One DKD step from snapshot timestep-1 into snapshot timestep (gravhopper.py:405-416)."""
        t = self.timestep
        dt = self._dt()
        x0, v0 = self._pos[t - 1], self._vel[t - 1]
        self._pos[t] = x0 + ((0.5 * v0) * dt) * U.KMS_MYR_TO_KPC
        kick_time = self._times[t - 1] + 0.5 * dt
        acc = np.asarray(U.value(self.calculate_acceleration(time=U.quantity(kick_time, U.TIME)),
                                 U.ACCEL, "acceleration"))
        self._vel[t] = v0 + acc * dt
        self._pos[t] = self._pos[t] + ((0.5 * self._vel[t]) * dt) * U.KMS_MYR_TO_KPC

    def calculate_acceleration(self, time=None):
        """N-body plus external acceleration at current_snap() (gravhopper.py:419-459)."""
        snap = self.current_snap()
        if self.Np > 1:
            if self.params["algorithm"] == "direct":
                nbody = jbgrav.direct_summation(snap, self.params["eps"], precision=self.params["precision"])
            elif self.params["algorithm"] == "tree":
                nbody = jbgrav.tree_force(snap, self.params["eps"], theta=self.params["theta"])
            else:
                raise UnknownAlgorithmException()
        else:
            nbody = U.quantity(np.zeros((self.Np, 3)), U.ACCEL)
        extra = self.calculate_extra_acceleration(snap["pos"], nbody, time=time,
                                                  vel=self.prev_snap()["vel"])
        return nbody + extra

    def calculate_extra_acceleration(self, pos, template_array, time=None, vel=None):
        """Sum of the registered external forces (gravhopper.py:462-473)."""
        ext = np.zeros_like(template_array)
        for fn, args in self.extra_force_functions:
            ext += fn(pos, args)
        for fn, args in self.extra_timedependent_force_functions:
            ext += fn(pos, time, args)
        for fn, args in self.extra_velocitydependent_force_functions:
            ext += fn(pos, vel, args)
        return ext

    # ---- external forces (gravhopper.py:603-845): plain callables -----------------
    # ``device=True`` (not in the reference) registers a DeviceForce: fn takes and
    # returns CUDA tensors and runs on the device-resident state.
    @staticmethod
    def _external(fn, device):
        if device:
            return fn if isinstance(fn, DeviceForce) else DeviceForce(fn)
        if not callable(fn):
            raise ExternalPackageException("Only callables are supported as external forces here.")
        return fn

    def add_external_force(self, fn, args=None, agama_units=None, device=False):
        """Add a position-dependent force ``fn(pos, args)`` (km/s/Myr when unitless)."""
        if isinstance(fn, list):
            for item in fn:
                self.add_external_force(item, args, device=device)
            return
        self.extra_force_functions.append((self._external(fn, device), args))

    def add_external_timedependent_force(self, fn, agama_units=None, args=None, device=False):
        """Add a time-dependent force ``fn(pos, time, args)``."""
        if isinstance(fn, list):
            for item in fn:
                self.add_external_timedependent_force(item, args=args, device=device)
            return
        self.extra_timedependent_force_functions.append((self._external(fn, device), args))

    def add_external_velocitydependent_force(self, fn, args=None, device=False):
        """Add a velocity-dependent force ``fn(pos, vel, args)``."""
        if isinstance(fn, list):
            for item in fn:
                self.add_external_velocitydependent_force(item, args, device=device)
            return
        self.extra_velocitydependent_force_functions.append((self._external(fn, device), args))

    # ---- initial conditions (gravhopper.py:848-904) --------------------------------
    def nrows(self, array):
        return array.shape[0] if np.ndim(array) > 1 else 1

    def add_IC(self, newIC):
        """Append particles: dict with 'pos', 'vel' (Np,3) and 'mass' (Np)."""
        if "pos" not in newIC:
            raise ICException("Missing 'pos' key in initial conditions function.")
        if "vel" not in newIC:
            raise ICException("Missing 'vel' key in initial conditions function.")
        if "mass" not in newIC:
            raise ICException("Missing 'mass' key in initial conditions function.")
        npos = self.nrows(newIC["pos"])
        nvel = self.nrows(newIC["vel"])
        nmass = len(newIC["mass"])
        if (npos != nvel) | (npos != nmass):
            raise ICException("Inconsistent number of particles in initial conditions function.")
        if self.ICarrays is False:
            self.ICarrays = {"pos": newIC["pos"], "vel": newIC["vel"], "mass": newIC["mass"]}
        else:
            self.ICarrays["pos"] = np.vstack((self.ICarrays["pos"], newIC["pos"]))
            self.ICarrays["vel"] = np.vstack((self.ICarrays["vel"], newIC["vel"]))
            self.ICarrays["mass"] = np.hstack((self.ICarrays["mass"], newIC["mass"]))


class IC(object):
    """Initial-condition generators (subset of gravhopper/gravhopper.py:1167-1734).

    Plain numbers are kpc, km/s, Msun.  Each returns {'pos', 'vel', 'mass'}.
    """

    @staticmethod
    def _finish(pos, vel, mass, center_pos, center_vel, force_origin):
        pos, vel = force_centers(pos, vel, center_pos, center_vel, force_origin)
        return {"pos": U.quantity(pos, U.LENGTH), "vel": U.quantity(vel, U.VELOCITY),
                "mass": U.quantity(mass, U.MASS)}

    @staticmethod
    def Plummer(N=None, b=None, totmass=None, center_pos=None, center_vel=None, force_origin=True,
                seed=None):
        """Isotropic Plummer sphere (gravhopper.py:1404-1493): speeds from q drawn by an
        inverse-CDF table of q^2 (1-q^2)^(7/2) on a 0.01 grid, as the reference does."""
        if N is None or b is None or totmass is None:
            raise ICException("Plummer requires N, b, and totmass.")
        b = float(U.value(b, U.LENGTH, "b"))
        M = float(U.value(totmass, U.MASS, "totmass"))
        rng = np.random.default_rng(seed)
        xi = rng.uniform(0.0, 1.0, size=N)
        r = b / np.sqrt(xi ** (-2.0 / 3) - 1)
        cth = rng.uniform(-1.0, 1.0, size=N)
        ph = rng.uniform(0.0, 2.0 * np.pi, size=N)
        sth = np.sqrt(1.0 - cth ** 2)
        pos = np.stack([r * sth * np.cos(ph), r * sth * np.sin(ph), r * cth], axis=1)
        qax = np.arange(0, 1.01, 0.01)
        cdf = np.cumsum(qax ** 2 * (1.0 - qax ** 2) ** 3.5)
        cdf /= cdf[-1]
        q = np.interp(rng.uniform(0.0, 1.0, size=N), cdf, qax)
        speed = q * np.sqrt(2.0 * U.G_KPC_KMS2_MSUN * M / b) * (1.0 + (r / b) ** 2) ** (-0.25)
        cvt = rng.uniform(-1.0, 1.0, size=N)
        vph = rng.uniform(0.0, 2.0 * np.pi, size=N)
        svt = np.sqrt(1.0 - cvt ** 2)
        vel = np.stack([speed * svt * np.cos(vph), speed * svt * np.sin(vph), speed * cvt], axis=1)
        return IC._finish(pos, vel, np.full(N, M / N), center_pos, center_vel, force_origin)

    @staticmethod
    def TSIS(N=None, maxrad=None, totmass=None, center_pos=None, center_vel=None, force_origin=True,
             seed=None):
        """Truncated singular isothermal sphere (gravhopper.py:1327-1400)."""
        if N is None or maxrad is None or totmass is None:
            raise ICException("TSIS requires N, maxrad, and totmass.")
        R = float(U.value(maxrad, U.LENGTH, "maxrad"))
        M = float(U.value(totmass, U.MASS, "totmass"))
        rng = np.random.default_rng(seed)
        sigma = np.sqrt(M * U.G_KPC_KMS2_MSUN / (2 * R))
        r = rng.uniform(0.0, R, size=N)
        cth = rng.uniform(-1.0, 1.0, size=N)
        ph = rng.uniform(0.0, 2.0 * np.pi, size=N)
        sth = np.sqrt(1.0 - cth ** 2)
        pos = np.stack([r * sth * np.cos(ph), r * sth * np.sin(ph), r * cth], axis=1)
        vel = np.stack([rng.normal(0.0, sigma, size=N) for _ in range(3)], axis=1)
        return IC._finish(pos, vel, np.full(N, M / N), center_pos, center_vel, force_origin)

    @staticmethod
    def Hernquist(N=None, a=None, totmass=None, cutoff=10.0, center_pos=None, center_vel=None,
                  force_origin=True, seed=None):
        """Hernquist sphere truncated at ``cutoff`` scale radii.  Velocities are Gaussian
        with the isotropic Jeans dispersion (the reference samples the distribution
        function instead, gravhopper.py:1497-1607)."""
        if N is None or a is None or totmass is None:
            raise ICException("Hernquist requires N, a, and totmass.")
        a = float(U.value(a, U.LENGTH, "a"))
        M = float(U.value(totmass, U.MASS, "totmass"))
        rng = np.random.default_rng(seed)
        xi = rng.uniform(0.0, cutoff ** 2 / (1.0 + cutoff) ** 2, size=N)
        r = a / (1.0 / np.sqrt(xi) - 1.0)
        cth = rng.uniform(-1.0, 1.0, size=N)
        ph = rng.uniform(0.0, 2.0 * np.pi, size=N)
        sth = np.sqrt(1.0 - cth ** 2)
        pos = np.stack([r * sth * np.cos(ph), r * sth * np.sin(ph), r * cth], axis=1)
        sig = np.sqrt(_ics.hernquist_sigma2(r, a, M))
        vel = sig[:, None] * rng.normal(size=(N, 3))
        return IC._finish(pos, vel, np.full(N, M / N), center_pos, center_vel, force_origin)

    @staticmethod
    def from_galpy_df(*args, **kwargs):
        raise ExternalPackageException("galpy is not available to use from_galpy_df()")

    @staticmethod
    def from_pyn_snap(*args, **kwargs):
        raise ExternalPackageException("Could not import pynbody to use from_pyn_snap()")


def force_centers(positions, velocities, center_pos=None, center_vel=None, force_origin=True):
    """Shift to the requested centre of mass and mean velocity (gravhopper.py:1740-1785)."""
    newpos = np.array(U.value(positions, U.LENGTH, "positions"), dtype=np.float64)
    newvel = np.array(U.value(velocities, U.VELOCITY, "velocities"), dtype=np.float64)
    if force_origin:
        if center_pos is None:
            center_pos = np.zeros(3)
        if center_vel is None:
            center_vel = np.zeros(3)
    if center_pos is not None:
        newpos += np.asarray(U.value(center_pos, U.LENGTH, "center_pos")) - newpos.mean(axis=0)
    if center_vel is not None:
        newvel += np.asarray(U.value(center_vel, U.VELOCITY, "center_vel")) - newvel.mean(axis=0)
    return newpos, newvel
