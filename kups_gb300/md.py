"""Fused Lennard-Jones molecular dynamics behind kUPS's ``Propagator`` interface.

Mirrors ``Propagator.__call__(key, state) -> state`` (src/kups/core/propagator.py:84-121)
for the propagators built by ``make_velocity_verlet_step``,
``make_baoab_langevin_step``, ``make_csvr_step`` and ``make_csvr_npt_step``
(src/kups/md/integrators.py:273-318, 405-455, 598-640, 801-890) around the
Lennard-Jones potential, as ``make_md_propagator`` wires them
(src/kups/application/md/simulation.py:74-119).  One call runs
``steps_per_call`` steps of every system in one persistent CUDA launch
(``kups_lj_md_run``).

State layout: the reference's particle table (float64 positions, momenta,
masses, species, system index; ``MDParticles``, application/md/data.py:31-65)
and system table (lattice ``tril``, time step, temperature, friction, CSVR and
barostat constants; ``MDSystems``, :68-106).  The NPT integrator scales the cell:
the returned state carries the new ``tril``.  Inside, atoms are packed once into float4 arrays
grouped by system (``PackedMD``); repeated calls on a ``PackedMD`` keep the
state on the device.  Capacity overflows restore the state from a backup and
retry with the size the kernel reported, as ``ResetOnErrorPropagator``
(propagator.py:534-566) with ``propagate_and_fix`` (:137-172) do.

Randomness: Philox4x32-10 keyed by (seed, atom) with the step as counter; the
JAX PRNG key is folded into the 64-bit seed (JAX's threefry stream cannot be
reproduced bit for bit, so stochastic parity is statistical).
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field, replace

import torch

from . import _lib
from .neighborlist import _stream, new_status, read_status
from .potential import LennardJonesParameters
from .units import BOLTZMANN_CONSTANT

INTEGRATORS = {"verlet": 0, "velocity_verlet": 0, "vv": 0, "nve": 0, "baoab": 1, "baoab_langevin": 1, "nvt": 1,
               "csvr": 2, "csvr_npt": 3, "npt": 3}


@dataclass
class MDParticles:
    positions: torch.Tensor  # f64 [N, 3]
    momenta: torch.Tensor  # f64 [N, 3]
    masses: torch.Tensor  # f64 [N]
    species: torch.Tensor  # int [N]
    system: torch.Tensor  # int [N]
    forces: torch.Tensor | None = None  # f64 [N, 3]; None = not yet computed


@dataclass
class MDSystems:
    tril: torch.Tensor  # f64 [S, 6]
    time_step: torch.Tensor  # [S] internal units (fs * FEMTO_SECOND)
    temperature: torch.Tensor  # [S] K
    friction_coefficient: torch.Tensor  # [S] 1 / internal time
    potential_energy: torch.Tensor | None = None
    kinetic_energy: torch.Tensor | None = None
    unitcell_gradients: torch.Tensor | None = None  # dE/dtril [S, 6]
    pressure: torch.Tensor | None = None  # instantaneous pressure [S] (energy / length^3)
    thermostat_time_constant: torch.Tensor | None = None  # [S] CSVR tau_T (internal time)
    target_pressure: torch.Tensor | None = None  # [S] P0 (energy / length^3)
    pressure_coupling_time: torch.Tensor | None = None  # [S] tau_P (internal time)
    compressibility: torch.Tensor | None = None  # [S] beta (length^3 / energy)
    minimum_scale_factor: torch.Tensor | None = None  # [S] barostat clip


@dataclass
class MDState:
    particles: MDParticles
    systems: MDSystems
    lj_parameters: LennardJonesParameters
    skin: float = 1.0
    step: int = 0


@dataclass
class PackedMD:
    """Device-resident packed state of a batch of systems."""

    pos4: torch.Tensor  # float32 [N, 4]
    mom4: torch.Tensor
    frc4: torch.Tensor
    perm: torch.Tensor  # int32 [N]: reference index of packed slot k
    sys_offset: torch.Tensor  # int32 [S + 1]
    order: torch.Tensor  # int32 [S], largest systems first
    tril32: torch.Tensor  # float32 [S, 6]
    cutoff: torch.Tensor  # float32 [S]
    skin: torch.Tensor
    dt: torch.Tensor
    kT: torch.Tensor
    friction: torch.Tensor
    lj_table: torch.Tensor  # float32 [T * T * 2]
    n_species: int
    max_atoms: int
    max_density: float
    max_range: float = 0.0  # largest cutoff + skin of the batch (host copy: no device read per launch)
    forces_valid: bool = False
    energy: torch.Tensor | None = None
    kinetic: torch.Tensor | None = None
    virial: torch.Tensor | None = None
    pressure: torch.Tensor | None = None
    rebuilds: torch.Tensor | None = None  # int32 [S], accumulated list builds (optional)
    profile: torch.Tensor | None = None  # int64 [10], cycles per kernel phase (optional)
    cell: torch.Tensor | None = None  # float64 [S, 6]: the cell the barostat scales
    thermostat_tau: torch.Tensor | None = None  # float64 [S] (CSVR, NPT)
    target_pressure: torch.Tensor | None = None  # float64 [S] (NPT)
    barostat_tau: torch.Tensor | None = None
    compressibility: torch.Tensor | None = None
    min_scale: torch.Tensor | None = None
    layout_key: tuple | None = None  # the inputs the layout fields were derived from (pack's reuse)

    @property
    def n_atoms(self) -> int:
        return self.pos4.shape[0]

    @property
    def n_systems(self) -> int:
        return self.sys_offset.shape[0] - 1

    def clone_dynamic(self) -> tuple:
        return (self.pos4.clone(), self.mom4.clone(), self.frc4.clone(),
                self.cell.clone() if self.cell is not None else None)

    def restore_dynamic(self, backup) -> None:
        self.pos4.copy_(backup[0])
        self.mom4.copy_(backup[1])
        self.frc4.copy_(backup[2])
        if backup[3] is not None:
            self.cell.copy_(backup[3])
            self.tril32.copy_(backup[3])


def lj_table(params: LennardJonesParameters) -> torch.Tensor:
    s = params.sigma.to(torch.float64)
    e = params.epsilon.to(torch.float64)
    return torch.stack([s * s, 4.0 * e], -1).reshape(-1).to(device="cuda", dtype=torch.float32)


def _layout_key(state: MDState) -> tuple:
    """The objects the packed layout and per-system parameters derive from, each with its
    tensor version counter: equal keys (same objects, unmodified) give equal layouts.  The
    key holds the objects, so their ids cannot be reused while it lives."""
    p, sy, lj = state.particles, state.systems, state.lj_parameters
    objs = (p.system, p.species, p.masses, sy.tril, sy.time_step, sy.temperature, sy.friction_coefficient,
            sy.thermostat_time_constant, sy.target_pressure, sy.pressure_coupling_time, sy.compressibility,
            sy.minimum_scale_factor, lj.sigma, lj.epsilon, lj.cutoff, state.skin)
    return tuple((o, o._version if isinstance(o, torch.Tensor) else None) for o in objs)


def _same_key(a: tuple | None, b: tuple) -> bool:
    return a is not None and len(a) == len(b) and all(x[0] is y[0] and x[1] == y[1] for x, y in zip(a, b))


def pack(state: MDState, reuse: PackedMD | None = None) -> PackedMD:
    """Reference layout -> packed device arrays (the kups_md_pack kernel).  With ``reuse`` a
    previous call's PackedMD whose layout key matches (same system, species, mass, cell and
    parameter objects, unmodified), the sort by system, offsets, queue order and per-system
    parameters are taken from it: only positions, momenta and forces are packed."""
    lib = _lib.load()
    p, sy = state.particles, state.systems
    dev = "cuda"
    key = _layout_key(state)
    if reuse is not None and _same_key(reuse.layout_key, key) and reuse.n_atoms == p.positions.shape[0]:
        n = reuse.n_atoms
        pos = p.positions.to(dev, torch.float64).contiguous()
        mom = p.momenta.to(dev, torch.float64).contiguous()
        frc = p.forces.to(dev, torch.float64).contiguous() if p.forces is not None else None
        mass = p.masses.to(dev, torch.float64).contiguous()
        species = p.species.to(dev, torch.int32).contiguous()
        pos4 = torch.empty((n, 4), device=dev, dtype=torch.float32)
        mom4 = torch.empty_like(pos4)
        frc4 = torch.empty_like(pos4)
        rc = lib.kups_md_pack(pos.data_ptr(), mom.data_ptr(), frc.data_ptr() if frc is not None else None,
                              mass.data_ptr(), species.data_ptr(), reuse.perm.data_ptr(), n, pos4.data_ptr(),
                              mom4.data_ptr(), frc4.data_ptr(), _stream())
        _lib.check(rc, "kups_md_pack")
        return replace(reuse, pos4=pos4, mom4=mom4, frc4=frc4, forces_valid=p.forces is not None,
                       energy=None, kinetic=None, virial=None, pressure=None, rebuilds=None, profile=None,
                       cell=sy.tril.to(dev, torch.float64).clone().contiguous(), layout_key=key)
    system = p.system.to(dev, torch.int64)
    n = system.shape[0]
    s = sy.tril.shape[0]
    perm = torch.argsort(system, stable=True)
    counts = torch.bincount(system, minlength=s)
    sys_offset = torch.zeros(s + 1, dtype=torch.int64, device=dev)
    sys_offset[1:] = torch.cumsum(counts, 0)
    order = torch.argsort(counts, descending=True, stable=True)
    pos = p.positions.to(dev, torch.float64).contiguous()
    mom = p.momenta.to(dev, torch.float64).contiguous()
    frc = p.forces.to(dev, torch.float64).contiguous() if p.forces is not None else None
    mass = p.masses.to(dev, torch.float64).contiguous()
    species = p.species.to(dev, torch.int32).contiguous()
    perm32 = perm.to(torch.int32).contiguous()
    pos4 = torch.empty((n, 4), device=dev, dtype=torch.float32)
    mom4 = torch.empty_like(pos4)
    frc4 = torch.empty_like(pos4)
    rc = lib.kups_md_pack(pos.data_ptr(), mom.data_ptr(), frc.data_ptr() if frc is not None else None,
                          mass.data_ptr(), species.data_ptr(), perm32.data_ptr(), n, pos4.data_ptr(),
                          mom4.data_ptr(), frc4.data_ptr(), _stream())
    _lib.check(rc, "kups_md_pack")
    f32 = lambda x: torch.as_tensor(x, dtype=torch.float64).to(dev).reshape(-1).expand(s).to(torch.float32).contiguous()
    tril = sy.tril.to(dev, torch.float64)
    vol = (tril[:, 0] * tril[:, 2] * tril[:, 5]).abs()
    dens = float((counts.to(torch.float64) / vol).max()) if s > 0 else 0.0
    kT = torch.as_tensor(sy.temperature, dtype=torch.float64).to(dev) * BOLTZMANN_CONSTANT
    f64 = lambda x: None if x is None else torch.as_tensor(x, dtype=torch.float64).to(dev).reshape(-1).expand(s).contiguous()
    cutoff32, skin32 = f32(state.lj_parameters.cutoff), f32(state.skin)
    rmax = float((cutoff32 + skin32).max()) if s > 0 else 0.0
    return PackedMD(
        pos4=pos4, mom4=mom4, frc4=frc4, perm=perm32, sys_offset=sys_offset.to(torch.int32).contiguous(),
        order=order.to(torch.int32).contiguous(), tril32=tril.to(torch.float32).contiguous(),
        cutoff=cutoff32, skin=skin32, dt=f32(sy.time_step), kT=f32(kT),
        friction=f32(sy.friction_coefficient), lj_table=lj_table(state.lj_parameters),
        n_species=int(state.lj_parameters.sigma.shape[0]), max_atoms=int(counts.max()) if s > 0 else 0,
        max_density=dens, max_range=rmax, forces_valid=p.forces is not None, cell=tril.clone().contiguous(),
        thermostat_tau=f64(sy.thermostat_time_constant), target_pressure=f64(sy.target_pressure),
        barostat_tau=f64(sy.pressure_coupling_time), compressibility=f64(sy.compressibility),
        min_scale=f64(sy.minimum_scale_factor), layout_key=key,
    )


def unpack(packed: PackedMD, state: MDState, integrator: int = 0) -> MDState:
    """Packed device arrays -> a new reference-layout state (kups_md_unpack)."""
    lib = _lib.load()
    n = packed.n_atoms
    pos = torch.empty((n, 3), device="cuda", dtype=torch.float64)
    mom = torch.empty_like(pos)
    frc = torch.empty_like(pos)
    rc = lib.kups_md_unpack(packed.pos4.data_ptr(), packed.mom4.data_ptr(), packed.frc4.data_ptr(),
                            packed.perm.data_ptr(), n, pos.data_ptr(), mom.data_ptr(), frc.data_ptr(), _stream())
    _lib.check(rc, "kups_md_unpack")
    parts = replace(state.particles, positions=pos, momenta=mom, forces=frc)
    systems = replace(state.systems, potential_energy=packed.energy, kinetic_energy=packed.kinetic,
                      unitcell_gradients=packed.virial, pressure=packed.pressure)
    if packed.cell is not None and integrator == INTEGRATORS["csvr_npt"]:
        systems = replace(systems, tril=packed.cell.clone())
    return replace(state, particles=parts, systems=systems)


def key_to_seed(key) -> int:
    if key is None:
        return 0
    if isinstance(key, int):
        return key & (2**64 - 1)
    t = torch.as_tensor(key).reshape(-1).to(torch.int64).cpu()
    h = 0x9E3779B97F4A7C15
    for v in t.tolist():
        h = ((h ^ (v & 0xFFFFFFFF)) * 0x100000001B3) & (2**64 - 1)
    return h


def run_bounds(system: torch.Tensor, n_systems: int, chunks: int) -> list[tuple[int, int, int, int]]:
    """Runs of whole systems for ``FusedLennardJonesMD.propagate_host``: (first atom, end atom,
    first system, end system) of each run.  A particle table grouped by system (non-decreasing
    ``system``) is cut at the system boundaries nearest to equal atom counts, each run keeping
    at least one atom; any other table is one run."""
    n = int(system.shape[0])
    counts = torch.bincount(system, minlength=n_systems) if n else torch.zeros(n_systems, dtype=torch.int64)
    offs = [0] + torch.cumsum(counts, 0).tolist()
    grouped = n == 0 or bool((system[1:] >= system[:-1]).all())
    cuts = [0]
    if grouped and chunks > 1 and n > 0:
        for k in range(1, chunks):
            target = k * n / chunks
            # the system boundary nearest the target that leaves atoms on both sides
            c = min((j for j in range(cuts[-1] + 1, n_systems) if offs[cuts[-1]] < offs[j] < n),
                    key=lambda j: abs(offs[j] - target), default=None)
            if c is not None:
                cuts.append(c)
    cuts.append(n_systems)
    return [(offs[s0], offs[s1], s0, s1) for s0, s1 in zip(cuts[:-1], cuts[1:])]


@dataclass
class _HostRun:
    """What ``FusedLennardJonesMD.propagate_host`` keeps between calls on one layout: the runs
    of whole systems (atom range, system range), a propagator per run, the runs' static
    device arrays (the same objects every call, so each run's packed layout is reused), the
    device buffers the host arrays are copied through, the copy stream and a second compute
    stream."""

    key: tuple
    chunks: int
    n: int
    bounds: list
    props: list
    static: list
    dev: list
    forces_host: torch.Tensor | None
    stream: torch.cuda.Stream  # host <-> device copies
    side: torch.cuda.Stream  # the second compute stream (odd runs)


@dataclass
class FusedLennardJonesMD:
    """Propagator: ``steps_per_call`` VV or BAOAB steps of LJ dynamics per call."""

    integrator: str = "baoab"
    steps_per_call: int = 1
    neighbor_capacity: int | None = None
    n_ctas: int = 0
    block_threads: int = 0
    min_lanes_per_atom: int = 0  # 0: library default; kups_gb300.autotune picks one per workload
    reuse_lists: bool = True  # resume systems whose workspace record matches the input (kups_md_args.reuse_lists)
    atom_base: int = 0  # global index of the first atom / system of this batch: the random streams
    system_base: int = 0  # are keyed by global indices (kups_md_args.atom_base / system_base)
    _ws: torch.Tensor | None = field(default=None, repr=False)
    _last: PackedMD | None = field(default=None, repr=False)
    _host: "_HostRun | None" = field(default=None, repr=False)

    def __call__(self, key, state: MDState) -> MDState:
        # the previous call's layout is reused while the state's system, cell and parameter
        # objects are the ones it was built from (the usual loop feeds each output back in)
        packed = pack(state, reuse=self._last)
        self._last = packed
        self.run_packed(packed, self.steps_per_call, key_to_seed(key), state.step)
        out = unpack(packed, state, INTEGRATORS[self.integrator])
        return replace(out, step=state.step + self.steps_per_call)

    def propagate_host(self, key, state: MDState, chunks: int = 4) -> MDState:
        """``__call__`` for a state whose positions, momenta and forces live in host memory
        (pinned, for the copies to overlap): those arrays are updated in place and returned in
        the new state, with the per-system outputs (energies, virial, pressure, the NPT cell)
        on the device.  When the particle table is grouped by system (non-decreasing
        ``system``), the batch is cut into ``chunks`` runs of whole systems of about equal atom
        counts, each with its own propagator, packed layout and workspace; the host-to-device
        copies of every run are queued at once on a copy stream, each run's launch waits only
        for its own inputs, and its results go back to the host while the next run computes.
        The random streams are keyed by the global atom and system index (``atom_base``,
        ``system_base``), so the result equals ``__call__`` on the same state bit for bit.
        Consecutive runs alternate between two compute streams, so a run's launch fills the SMs
        that the previous run's last systems leave idle.
        Static arrays (masses, species, system index, the system table) may live on the host
        or the device; keeping the same objects between calls keeps the packed layouts and the
        resumable Verlet lists.  Returns after the results are in host memory and every run's
        status is checked (capacity overflows are retried run by run, as ``run_packed`` does)."""
        p = state.particles
        if p.positions.is_cuda or p.momenta.is_cuda or (p.forces is not None and p.forces.is_cuda):
            raise ValueError("propagate_host takes positions, momenta and forces in host memory")
        run = self._host_run(state, int(chunks))
        seed, step0, integ = key_to_seed(key), state.step, INTEGRATORS[self.integrator]
        comp, copy = torch.cuda.current_stream(), run.stream
        have_f = p.forces is not None
        if not have_f and (run.forces_host is None or run.forces_host.shape != p.positions.shape):
            run.forces_host = torch.zeros(p.positions.shape, dtype=torch.float64).pin_memory()
        frc_h = p.forces if have_f else run.forces_host
        ev_in = []
        with torch.cuda.stream(copy):
            copy.wait_stream(comp)  # the device buffers of the previous call are free
            for (a0, a1, _, _), (dp, dm, df) in zip(run.bounds, run.dev):
                dp.copy_(p.positions[a0:a1], non_blocking=True)
                dm.copy_(p.momenta[a0:a1], non_blocking=True)
                if have_f:
                    df.copy_(p.forces[a0:a1], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(copy)
                ev_in.append(ev)
        done = []
        # consecutive runs alternate between two compute streams: the next run's CTAs take the
        # SMs the previous run's last systems leave idle (each run is one persistent launch)
        streams = (comp, run.side)
        run.side.wait_stream(comp)
        for k, ((a0, a1, _, _), (dp, dm, df), sub, stat) in enumerate(zip(run.bounds, run.dev, run.props, run.static)):
            self._sync_settings(sub)
            with torch.cuda.stream(streams[k % 2]):
                torch.cuda.current_stream().wait_event(ev_in[k])
                st_k = MDState(MDParticles(dp, dm, stat[0], stat[1], stat[2], df if have_f else None), stat[3],
                               state.lj_parameters, skin=state.skin, step=step0)
                packed = pack(st_k, reuse=sub._last)
                sub._last = packed
                backup, valid0 = packed.clone_dynamic(), packed.forces_valid
                status = sub.launch(packed, self.steps_per_call, seed, step0)
                out = unpack(packed, st_k, integ)
                self._to_host(run, out, p.positions, p.momenta, frc_h, a0, a1)
            done.append([packed, backup, valid0, status, st_k, out])
        comp.wait_stream(run.side)
        comp.wait_stream(copy)
        comp.synchronize()
        for k, (packed, backup, valid0, status, st_k, out) in enumerate(done):
            code = read_status(status)
            if code.code == _lib.KUPS_OK:
                continue
            if code.code != _lib.KUPS_ERR_CAPACITY or code.detail != _lib.KUPS_CAP_NEIGHBORS:
                _lib.raise_status(code)
            sub, (a0, a1, _, _) = run.props[k], run.bounds[k]
            packed.restore_dynamic(backup)
            packed.forces_valid = valid0
            sub.neighbor_capacity = int(math.ceil(code.required * 1.25 / 16.0) * 16)
            sub.run_packed(packed, self.steps_per_call, seed, step0)
            out = unpack(packed, st_k, integ)
            self._to_host(run, out, p.positions, p.momenta, frc_h, a0, a1)
            comp.wait_stream(copy)
            comp.synchronize()
            done[k][5] = out
        cat = lambda xs: None if any(x is None for x in xs) else torch.cat(xs)
        outs = [d[5].systems for d in done]
        systems = replace(state.systems, potential_energy=cat([o.potential_energy for o in outs]),
                          kinetic_energy=cat([o.kinetic_energy for o in outs]),
                          unitcell_gradients=cat([o.unitcell_gradients for o in outs]),
                          pressure=cat([o.pressure for o in outs]))
        if integ == INTEGRATORS["csvr_npt"]:
            systems = replace(systems, tril=torch.cat([o.tril for o in outs]))
        return replace(state, particles=replace(p, forces=frc_h), systems=systems,
                       step=step0 + self.steps_per_call)

    @staticmethod
    def _to_host(run, out: MDState, pos_h, mom_h, frc_h, a0: int, a1: int) -> None:
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream())
        with torch.cuda.stream(run.stream):
            run.stream.wait_event(ev)
            for t, h in ((out.particles.positions, pos_h), (out.particles.momenta, mom_h),
                         (out.particles.forces, frc_h)):
                t.record_stream(run.stream)
                h[a0:a1].copy_(t, non_blocking=True)

    def _sync_settings(self, sub: "FusedLennardJonesMD") -> None:
        sub.integrator, sub.steps_per_call = self.integrator, self.steps_per_call
        sub.n_ctas, sub.block_threads = self.n_ctas, self.block_threads
        sub.min_lanes_per_atom, sub.reuse_lists = self.min_lanes_per_atom, self.reuse_lists
        if self.neighbor_capacity is not None:
            sub.neighbor_capacity = self.neighbor_capacity

    def _host_run(self, state: MDState, chunks: int) -> "_HostRun":
        key = _layout_key(state)
        p, sy = state.particles, state.systems
        n, s = int(p.positions.shape[0]), int(sy.tril.shape[0])
        run = self._host
        if run is not None and run.chunks == chunks and run.n == n and _same_key(run.key, key):
            return run
        bounds = run_bounds(p.system.to("cpu", torch.int64), s, chunks)
        dev = "cuda"
        masses, species = p.masses.to(dev), p.species.to(dev)
        system_d = p.system.to(dev)
        old = {(b[0], b[2]): q for b, q in zip(run.bounds, run.props)} if run is not None else {}
        props, static, bufs = [], [], []
        for a0, a1, s0, s1 in bounds:
            sub = old.get((a0, s0)) or FusedLennardJonesMD(atom_base=a0, system_base=s0)
            sub.atom_base, sub.system_base = a0, s0
            props.append(sub)
            cut = lambda x: x[s0:s1] if isinstance(x, torch.Tensor) and x.dim() > 0 and x.shape[0] == s else x
            sys_k = MDSystems(**{f: (cut(getattr(sy, f)).to(dev) if isinstance(getattr(sy, f), torch.Tensor)
                                     else getattr(sy, f)) for f in sy.__dataclass_fields__})
            static.append((masses[a0:a1], species[a0:a1], (system_d[a0:a1] - s0), sys_k))
            bufs.append(tuple(torch.empty((a1 - a0, 3), device=dev, dtype=torch.float64) for _ in range(3)))
        stream = run.stream if run is not None else torch.cuda.Stream()
        side = run.side if run is not None else torch.cuda.Stream()
        fh = run.forces_host if run is not None else None
        self._host = _HostRun(key=key, chunks=chunks, n=n, bounds=bounds, props=props, static=static, dev=bufs,
                              forces_host=fh, stream=stream, side=side)
        return self._host

    def capacity_for(self, packed: PackedMD) -> int:
        if self.neighbor_capacity is not None:
            return self.neighbor_capacity
        rl = packed.max_range if packed.max_range > 0 else float((packed.cutoff + packed.skin).max())
        est = 4.0 / 3.0 * math.pi * rl**3 * packed.max_density * 1.35 + 16
        return int(math.ceil(est / 16.0) * 16)

    def args(self, packed: PackedMD, n_steps: int, seed: int, step0: int, trace_pe=None, trace_ke=None,
             virial: bool = True, trace_virial=None) -> _lib.MdArgs:
        s = packed.n_systems
        if packed.energy is None:
            packed.energy = torch.zeros(s, device="cuda", dtype=torch.float64)
            packed.kinetic = torch.zeros(s, device="cuda", dtype=torch.float64)
            packed.virial = torch.zeros((s, 6), device="cuda", dtype=torch.float64)
            packed.pressure = torch.zeros(s, device="cuda", dtype=torch.float64)
        a = _lib.MdArgs()
        a.pos, a.mom, a.force = packed.pos4.data_ptr(), packed.mom4.data_ptr(), packed.frc4.data_ptr()
        a.sys_offset, a.order, a.tril = packed.sys_offset.data_ptr(), packed.order.data_ptr(), packed.tril32.data_ptr()
        a.cutoff, a.skin, a.dt = packed.cutoff.data_ptr(), packed.skin.data_ptr(), packed.dt.data_ptr()
        a.kT, a.friction, a.lj_table = packed.kT.data_ptr(), packed.friction.data_ptr(), packed.lj_table.data_ptr()
        a.energy, a.kinetic = packed.energy.data_ptr(), packed.kinetic.data_ptr()
        a.virial = packed.virial.data_ptr() if virial else None
        a.pressure = packed.pressure.data_ptr() if virial and packed.pressure is not None else None
        a.trace_pe = trace_pe.data_ptr() if trace_pe is not None else None
        a.trace_ke = trace_ke.data_ptr() if trace_ke is not None else None
        a.trace_virial = trace_virial.data_ptr() if trace_virial is not None else None
        a.rebuilds = packed.rebuilds.data_ptr() if packed.rebuilds is not None else None
        a.profile = packed.profile.data_ptr() if packed.profile is not None else None
        a.n_atoms, a.n_systems, a.n_species = packed.n_atoms, s, packed.n_species
        a.n_steps = int(n_steps)
        a.integrator = INTEGRATORS[self.integrator]
        a.forces_valid = int(packed.forces_valid)
        a.neighbor_capacity = self.capacity_for(packed)
        a.seed, a.step0 = int(seed) & (2**64 - 1), int(step0)
        a.n_ctas, a.block_threads = self.n_ctas, self.block_threads
        a.min_lanes_per_atom = self.min_lanes_per_atom
        a.reuse_lists = int(bool(self.reuse_lists))
        a.atom_base, a.system_base = int(self.atom_base), int(self.system_base)
        if a.integrator >= 2:
            need = ["thermostat_tau"] + (["target_pressure", "barostat_tau", "compressibility", "min_scale"]
                                         if a.integrator == 3 else [])
            missing = [k for k in need if getattr(packed, k) is None]
            if missing:
                raise ValueError(f"integrator {self.integrator!r} needs the system fields {missing}")
            a.thermostat_tau = packed.thermostat_tau.data_ptr()
            if a.integrator == 3:
                a.target_pressure, a.barostat_tau = packed.target_pressure.data_ptr(), packed.barostat_tau.data_ptr()
                a.compressibility, a.min_scale = packed.compressibility.data_ptr(), packed.min_scale.data_ptr()
                a.cell = packed.cell.data_ptr()
        return a

    def workspace(self, a: _lib.MdArgs) -> torch.Tensor:
        nbytes = _lib.load().kups_lj_md_workspace_bytes(C.byref(a))
        if self._ws is None or self._ws.numel() < nbytes:
            # the per-system records start invalid (a record is trusted only after exact checks,
            # zeros make the first call skip them outright)
            self._ws = torch.zeros(nbytes, device="cuda", dtype=torch.uint8)
        return self._ws

    def launch(self, packed: PackedMD, n_steps: int, seed: int = 0, step0: int = 0, status=None, trace_pe=None,
               trace_ke=None, virial: bool = True, trace_virial=None) -> torch.Tensor:
        """Enqueue one persistent launch (no host synchronisation).  trace_pe / trace_ke
        [n_steps, S] and trace_virial [n_steps, S, 6] (float64, optional) receive the potential
        energy, kinetic energy and dE/dtril after every step."""
        a = self.args(packed, n_steps, seed, step0, trace_pe, trace_ke, virial, trace_virial)
        ws = self.workspace(a)
        status = status if status is not None else new_status()
        rc = _lib.load().kups_lj_md_run(C.byref(a), ws.data_ptr(), ws.numel(), status.data_ptr(), _stream())
        _lib.check(rc, "kups_lj_md_run")
        packed.forces_valid = True
        if a.integrator == 3:
            packed.tril32.copy_(packed.cell)
        return status

    def run_packed(self, packed: PackedMD, n_steps: int, seed: int = 0, step0: int = 0, trace: bool = False,
                   max_tries: int = 6):
        """Run and check the status; on a capacity overflow restore and retry."""
        backup = packed.clone_dynamic()
        valid0 = packed.forces_valid
        for _ in range(max_tries):
            tpe = tke = None
            if trace:
                tpe = torch.zeros((n_steps, packed.n_systems), device="cuda", dtype=torch.float64)
                tke = torch.zeros_like(tpe)
            st = self.launch(packed, n_steps, seed, step0, None, tpe, tke)
            status = read_status(st)
            if status.code == _lib.KUPS_OK:
                return (tpe, tke) if trace else None
            if status.code == _lib.KUPS_ERR_CAPACITY and status.detail == _lib.KUPS_CAP_NEIGHBORS:
                packed.restore_dynamic(backup)
                packed.forces_valid = valid0
                self.neighbor_capacity = int(math.ceil(status.required * 1.25 / 16.0) * 16)
                continue
            _lib.raise_status(status)
        raise _lib.KupsError("fused MD capacity did not converge")


def make_velocity_verlet_step(steps_per_call: int = 1, **kw) -> FusedLennardJonesMD:
    """Velocity Verlet (NVE) with the LJ force as derivative computation (integrators.py:273-318)."""
    return FusedLennardJonesMD("velocity_verlet", steps_per_call, **kw)


def make_baoab_langevin_step(steps_per_call: int = 1, **kw) -> FusedLennardJonesMD:
    """BAOAB Langevin (NVT) with the LJ force as derivative computation (integrators.py:405-455)."""
    return FusedLennardJonesMD("baoab", steps_per_call, **kw)


def make_csvr_step(steps_per_call: int = 1, **kw) -> FusedLennardJonesMD:
    """CSVR thermostat then velocity Verlet (NVT; integrators.py:598-640); needs
    ``MDSystems.thermostat_time_constant``."""
    return FusedLennardJonesMD("csvr", steps_per_call, **kw)


def make_csvr_npt_step(steps_per_call: int = 1, **kw) -> FusedLennardJonesMD:
    """CSVR, velocity Verlet, stochastic cell rescaling and the forces again (NPT;
    integrators.py:801-890); needs the thermostat and barostat system fields."""
    return FusedLennardJonesMD("csvr_npt", steps_per_call, **kw)


class LennardJonesMD64:
    """Float64 LJ molecular dynamics: the reference's own arithmetic, step by step.

    One step is the reference's propagator (``make_velocity_verlet_step`` / ``make_baoab_langevin_step``,
    src/kups/md/integrators.py:273-318, 405-455) with its derivative computation as the reference's MD
    application runs it (application/md/simulation.py:74-119): the neighbour list rebuilt at every step
    (``kups_neighborlist_build``, exact float64 membership), LJ energy and gradients over the edges in
    float64 (``kups_lj_edges``), and the float64 integrator blocks (``kups_md_kick`` / ``kups_md_drift``
    with the wrap / ``kups_md_thermostat``).  Every launch is stream-ordered with no host
    synchronisation; velocity-Verlet steps replay from one captured CUDA graph.  This is the float64
    counterpart of ``FusedLennardJonesMD`` (float32 pair arithmetic), for small systems that must
    match the reference's float64 trajectory.
    """

    def __init__(self, state: MDState, integrator: str = "baoab", avg_edges: int | None = None, seed: int = 0):
        from .neighborlist import _f64, _i32

        if INTEGRATORS[integrator] not in (0, 1):
            raise ValueError("LennardJonesMD64 runs velocity Verlet or BAOAB")
        self.integrator = INTEGRATORS[integrator]
        p, sy = state.particles, state.systems
        self.pos = _f64(p.positions).clone()
        self.mom = _f64(p.momenta).clone()
        self.mass = _f64(p.masses)
        self.species = _i32(p.species)
        self.system = _i32(p.system)
        self.tril = _f64(sy.tril).reshape(-1, 6).contiguous()
        s = self.tril.shape[0]
        self.s, self.n = s, self.pos.shape[0]
        full = lambda x: _f64(torch.as_tensor(x, dtype=torch.float64).reshape(-1).expand(s))
        self.dt = full(sy.time_step)
        self.kT = full(torch.as_tensor(sy.temperature, dtype=torch.float64) * BOLTZMANN_CONSTANT)
        self.friction = full(sy.friction_coefficient)
        prm = state.lj_parameters
        self.cut = full(prm.cutoff)
        self.sig, self.eps = _f64(prm.sigma), _f64(prm.epsilon)
        self.nsp = int(self.sig.shape[0])
        if avg_edges is None:
            vol = float((self.tril[:, 0] * self.tril[:, 2] * self.tril[:, 5]).abs().min())
            counts = torch.bincount(self.system.long(), minlength=s)
            dens = float(counts.max()) / vol
            avg_edges = int(4.0 / 3.0 * math.pi * float(self.cut.max()) ** 3 * dens * 1.5) + 32
        self.cap = int(avg_edges) * self.n
        dev = dict(device="cuda")
        self.edges = torch.empty((self.cap, 2), dtype=torch.int32, **dev)
        self.shifts = torch.empty((self.cap, 3), dtype=torch.int32, **dev)
        self.n_edges = torch.zeros(1, dtype=torch.int64, **dev)
        self.incl = self.system
        self.excl = torch.arange(self.n, dtype=torch.int32, **dev)
        lib = _lib.load()
        self.nl_ws = torch.empty(lib.kups_neighborlist_workspace_bytes(self.n, s), dtype=torch.uint8, **dev)
        self.energy = torch.zeros(s, dtype=torch.float64, **dev)
        self.grad = torch.zeros((self.n, 3), dtype=torch.float64, **dev)
        self.gtril = torch.zeros((s, 6), dtype=torch.float64, **dev)
        self.status = new_status()
        self.seed = int(seed)
        self.step = int(state.step)
        # the Langevin noise counter lives on the device, so a captured step replays as the next one
        self.counter = torch.tensor([self.step], dtype=torch.int64, device="cuda")
        self.graph = None
        self._forces()

    def _forces(self):
        lib = _lib.load()
        st = _stream()
        rc = lib.kups_neighborlist_build(self.pos.data_ptr(), self.system.data_ptr(), self.incl.data_ptr(),
                                         self.excl.data_ptr(), self.n, self.s, self.tril.data_ptr(),
                                         self.cut.data_ptr(), self.s, self.edges.data_ptr(), self.shifts.data_ptr(),
                                         self.cap, self.n_edges.data_ptr(), self.nl_ws.data_ptr(), self.nl_ws.numel(),
                                         self.status.data_ptr(), st)
        _lib.check(rc, "kups_neighborlist_build")
        # edges past n_edges are padded with the out-of-bounds index and skipped by the kernel
        rc = lib.kups_lj_edges(self.pos.data_ptr(), self.system.data_ptr(), self.species.data_ptr(), self.n,
                               self.tril.data_ptr(), self.cut.data_ptr(), self.s, self.sig.data_ptr(),
                               self.eps.data_ptr(), self.nsp, self.edges.data_ptr(), self.shifts.data_ptr(), self.cap,
                               self.energy.data_ptr(), self.grad.data_ptr(), self.gtril.data_ptr(), 0,
                               self.status.data_ptr(), st)
        _lib.check(rc, "kups_lj_edges")

    def _step(self, step: int):
        lib = _lib.load()
        st = _stream()
        args = (self.pos.data_ptr(), self.mom.data_ptr(), self.mass.data_ptr(), self.system.data_ptr(),
                self.dt.data_ptr(), self.tril.data_ptr())
        lib.kups_md_kick(self.mom.data_ptr(), self.grad.data_ptr(), self.system.data_ptr(), self.dt.data_ptr(), 0.5,
                         self.n, st)
        if self.integrator == 1:
            lib.kups_md_drift(*args, 0.5, self.n, st)
            lib.kups_md_thermostat_counted(self.mom.data_ptr(), self.mass.data_ptr(), self.system.data_ptr(),
                                           self.dt.data_ptr(), self.kT.data_ptr(), self.friction.data_ptr(),
                                           self.seed, self.counter.data_ptr(), self.n, st)
            self.counter.add_(1)
            lib.kups_md_drift(*args, 0.5, self.n, st)
        else:
            lib.kups_md_drift(*args, 1.0, self.n, st)
        self._forces()
        lib.kups_md_kick(self.mom.data_ptr(), self.grad.data_ptr(), self.system.data_ptr(), self.dt.data_ptr(), 0.5,
                         self.n, st)

    def run(self, n_steps: int, use_graph: bool = True):
        """n_steps steps (the Langevin noise of step k is keyed by (seed, atom, k)); after a warm-up
        step the step is captured once as a CUDA graph and replayed."""
        if not use_graph:
            for _ in range(n_steps):
                self._step(self.step)
                self.step += 1
            return
        if self.graph is None and n_steps > 0:
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                self._step(self.step)
            torch.cuda.current_stream().wait_stream(s)
            self.step += 1
            n_steps -= 1
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph):
                self._step(0)
        for _ in range(max(n_steps, 0)):
            self.graph.replay()
            self.step += 1

    def check(self):
        _lib.raise_status(read_status(self.status))

    def kinetic_energy(self) -> torch.Tensor:
        ke = 0.5 * (self.mom**2).sum(-1) / self.mass
        return torch.zeros(self.s, dtype=torch.float64, device="cuda").index_add_(0, self.system.long(), ke)
