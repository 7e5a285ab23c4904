"""pimc_gb300 — Python host binding of the GB300 PIMC engine's C ABI.

The engine (libpimc_gb300.so, built by ``pimc_gb300.build``) runs pi-qmc's
multilevel-bisection hot path on an sm_103a GPU.  This module is a thin ctypes
layer over include/pimc_gb300.h; names follow pi-qmc (SimulationInfo fields,
getActionDifference, NodeModel::evaluate, ThermoEnergyEstimator).  There is no
CPU fallback: without the library or a GPU every call raises.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB
MAXS = 4
MAXL = 6
PIMC_NODES_NONE, PIMC_NODES_SHO, PIMC_NODES_FREE = 0, 1, 2
PIMC_MOVER_FREE, PIMC_MOVER_FREE_PBC = 0, 1
PIMC_PREC_FP64, PIMC_PREC_MIXED = 0, 1
PIMC_ERR_INVALID, PIMC_ERR_CUDA, PIMC_ERR_NO_DEVICE, PIMC_ERR_CAPACITY = -1, -2, -3, -4
PIMC_STATUS_INIT_CROSSING, PIMC_STATUS_SINGULAR = 1, 2
PIMC_STATUS_RESCALE_LIMIT, PIMC_STATUS_NONFINITE = 4, 8
STATUS_BITS = {1: "init_crossing", 2: "singular", 4: "rescale_limit", 8: "nonfinite"}


class PimcError(RuntimeError):
    pass


class System(C.Structure):
    """pimc_system: one simulated system (SimulationInfo + action attributes)."""
    _fields_ = [
        ("npart", C.c_int), ("nspecies", C.c_int),
        ("spec_count", C.c_int * MAXS), ("spec_mass", C.c_double * MAXS),
        ("spec_charge", C.c_double * MAXS), ("sho_omega", C.c_double * MAXS),
        ("prim_a", C.c_double * MAXS), ("prim_b", C.c_double * MAXS),
        ("node_kind", C.c_int * MAXS), ("node_omega", C.c_double * MAXS),
        ("node_temperature", C.c_double), ("nslice", C.c_int), ("tau", C.c_double),
        ("nlevel", C.c_int), ("cell", C.c_double * 3), ("spring", C.c_int),
        ("coulomb", C.c_int), ("epsilon", C.c_double), ("ewald", C.c_int), ("mover", C.c_int),
        ("delayed_rejection", C.c_int), ("sigma_factor", C.c_double),
        ("dr_sigma_factor", C.c_double),
    ]


class PairTable(C.Structure):
    _fields_ = [("species1", C.c_int), ("species2", C.c_int), ("ngpts", C.c_int),
                ("norder", C.c_int), ("rgridinv", C.c_double), ("logrratioinv", C.c_double),
                ("ugrid", C.POINTER(C.c_double))]


class EwaldTable(C.Structure):
    _fields_ = [("totk", C.c_int), ("kvec", C.POINTER(C.c_int)), ("vk", C.POINTER(C.c_double)),
                ("one_over_2v", C.c_double), ("self_energy", C.c_double), ("ikmax", C.c_int * 3)]


class LaunchConfig(C.Structure):
    _fields_ = [("block", C.c_int), ("scratch_global", C.c_int), ("ctas_per_sm", C.c_int),
                ("regs_variant", C.c_int), ("ms", C.c_float)]

    def as_dict(self):
        return {"block": self.block, "scratch_global": self.scratch_global,
                "ctas_per_sm": self.ctas_per_sm, "regs_variant": self.regs_variant,
                "ms": round(float(self.ms), 4)}


class DisplaceRecord(C.Structure):
    _fields_ = [("ipart", C.c_int * 4), ("disp", (C.c_double * 3) * 4), ("ds", C.c_double),
                ("ds_node", C.c_double), ("accepted", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int), ("hbm_bytes", C.c_size_t), ("max_npart", C.c_int),
                ("max_nslice", C.c_int), ("max_level", C.c_int), ("max_node_count", C.c_int)]


class ReplicaState(C.Structure):
    _fields_ = [("attempt", C.c_uint32), ("status", C.c_uint32), ("accepted", C.c_int64),
                ("attempted", C.c_int64), ("node_scale", C.c_double * 4)]

    def as_dict(self):
        return {"attempt": self.attempt, "status": self.status, "accepted": self.accepted,
                "attempted": self.attempted, "node_scale": list(self.node_scale)}

    @classmethod
    def from_dict(cls, d):
        st = cls()
        st.attempt, st.status = d["attempt"], d["status"]
        st.accepted, st.attempted = d["accepted"], d["attempted"]
        for k, v in enumerate(d["node_scale"]):
            st.node_scale[k] = v
        return st


class MoveRecord(C.Structure):
    _fields_ = [("ifirst1", C.c_int), ("ifirst2", C.c_int), ("ipart", C.c_int),
                ("reject_level", C.c_int), ("ds", C.c_double * (MAXL + 3)),
                ("ds_node", C.c_double * (MAXL + 3)), ("lnt", C.c_double * (MAXL + 3))]


def system_from_kw(kw):
    """A pimc_system from workload keywords (see pimc_gb300.workloads)."""
    s = System()
    counts = kw["counts"]
    ns = len(counts)
    s.nspecies = ns
    s.npart = int(sum(counts))
    get = lambda k, d: kw.get(k, [d] * ns)  # noqa: E731
    for i in range(ns):
        s.spec_count[i] = counts[i]
        s.spec_mass[i] = get("masses", 1.0)[i]
        s.spec_charge[i] = get("charges", -1.0)[i]
        s.sho_omega[i] = get("sho_omega", 0.0)[i]
        s.prim_a[i] = get("prim_a", 0.0)[i]
        s.prim_b[i] = get("prim_b", 0.0)[i]
        s.node_kind[i] = get("node_kind", 0)[i]
        s.node_omega[i] = get("node_omega", 0.0)[i]
    s.nslice = kw["nslice"]
    s.tau = kw["beta"] / kw["nslice"]
    s.node_temperature = kw.get("node_temperature", 1.0 / kw["beta"])
    s.nlevel = kw["nlevel"]
    cell = kw.get("cell", 1000.0)
    cell = cell if hasattr(cell, "__len__") else [cell] * 3
    for d in range(3):
        s.cell[d] = cell[d]
    s.spring = kw.get("spring", 1)
    s.coulomb = kw.get("coulomb", 0)
    s.epsilon = kw.get("epsilon", 1.0)
    s.ewald = kw.get("ewald", 0)
    s.mover = kw.get("mover", 0)
    # <Sample delayedRejection defaultSigmaFactor newSigmaFactor> (0: pi-qmc's defaults)
    s.delayed_rejection = int(kw.get("delayed_rejection", 0))
    s.sigma_factor = kw.get("sigma_factor", 0.0)
    s.dr_sigma_factor = kw.get("dr_sigma_factor", 0.0)
    return s


_lib = None


def lib():
    """Load the engine library (fails loudly if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PimcError(f"engine library not built: {LIB_PATH} (run pimc_gb300.build)")
        L = C.CDLL(LIB_PATH)
        P, I, D = C.c_void_p, C.c_int, C.POINTER(C.c_double)
        L.pimc_last_error.restype = C.c_char_p
        L.pimc_engine_create.argtypes = [C.POINTER(System), I, C.POINTER(PairTable), I,
                                         C.POINTER(EwaldTable), C.c_uint64, I, C.POINTER(P)]
        L.pimc_engine_create_batch.argtypes = [C.POINTER(System), I, C.POINTER(PairTable),
                                               C.POINTER(C.c_int), C.c_uint64, I, C.POINTER(P)]
        L.pimc_engine_destroy.argtypes = [P]
        L.pimc_set_stream.argtypes = [P, P]
        L.pimc_upload_paths.argtypes = [P, D]
        L.pimc_download_paths.argtypes = [P, D]
        L.pimc_path_offsets.argtypes = [P, C.POINTER(C.c_int64)]
        L.pimc_run_sections.argtypes = [P, I, C.POINTER(MoveRecord)]
        L.pimc_replica_status.argtypes = [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                          C.POINTER(C.c_uint32)]
        L.pimc_thermo_energy.argtypes = [P, D]
        L.pimc_run_steps.argtypes = [P, I, I, D]
        L.pimc_virial_energy.argtypes = [P, I, D]
        L.pimc_run_displace.argtypes = [P, I, D, I, I, C.POINTER(DisplaceRecord)]
        L.pimc_coulomb_energy.argtypes = [P, C.c_double, D]
        L.pimc_ewald_coulomb_energy.argtypes = [P, C.c_double, C.c_double,
                                                C.POINTER(EwaldTable), D, D]
        L.pimc_ewald_estimator_tables.argtypes = [C.POINTER(System), C.c_double, C.c_double,
                                                  C.c_double, C.POINTER(C.POINTER(EwaldTable)),
                                                  D]
        L.pimc_action_difference.argtypes = [P, I, I, D, D, C.POINTER(C.c_int), D]
        L.pimc_node_evaluate.argtypes = [P, I, I, D, D, D, D, D, C.POINTER(C.c_int)]
        L.pimc_node_scale.argtypes = [P, I, I, D]
        L.pimc_stream_sample.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, I, D, D]
        L.pimc_fp64_peak.argtypes = [D]
        L.pimc_fp32_peak.argtypes = [D]
        L.pimc_node_evaluate_noalloc.argtypes = [C.POINTER(System), I, C.c_double, I, P, P, P,
                                                 P, P, P, P]
        L.pimc_engine_configure.argtypes = [P, C.POINTER(LaunchConfig)]
        L.pimc_engine_get_config.argtypes = [P, C.POINTER(LaunchConfig)]
        L.pimc_engine_autotune.argtypes = [P, I, C.POINTER(LaunchConfig),
                                           C.POINTER(LaunchConfig), I, C.POINTER(C.c_int)]
        L.pimc_server_create.argtypes = [C.POINTER(ServerConfig), C.c_uint64, I, C.POINTER(P)]
        L.pimc_server_admit.argtypes = [P, C.POINTER(System), C.POINTER(PairTable), I, D,
                                        C.c_uint32, I, C.POINTER(C.c_int)]
        L.pimc_server_release.argtypes = [P, I]
        L.pimc_server_run.argtypes = [P]
        L.pimc_server_energy.argtypes = [P, D]
        L.pimc_server_energy_slots.argtypes = [P, C.POINTER(C.c_int), I, D]
        L.pimc_server_download_path.argtypes = [P, I, D]
        L.pimc_server_pool.argtypes = [P, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
        L.pimc_kernel_launches.argtypes = [P]
        L.pimc_kernel_launches.restype = C.c_int64
        L.pimc_paths_write_file.argtypes = [C.c_char_p, D, I, I]
        L.pimc_paths_read_file.argtypes = [C.c_char_p, D, I, I, I]
        L.pimc_write_paths.argtypes = [P, I, C.c_char_p]
        L.pimc_read_paths.argtypes = [P, I, C.c_char_p, I]
        L.pimc_get_replica_state.argtypes = [P, I, C.POINTER(ReplicaState)]
        L.pimc_set_replica_state.argtypes = [P, I, C.POINTER(ReplicaState)]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise PimcError(f"pimc error {rc}: {lib().pimc_last_error().decode()}")


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def write_paths_file(filename, xyz):
    """One path [nslice][npart][3] to a file in pi-qmc's restart format
    (WritePaths, src/algorithm/WritePaths.cc:25-114)."""
    x = np.ascontiguousarray(xyz, np.float64)
    _check(lib().pimc_paths_write_file(os.fsencode(filename), _dp(x), x.shape[1], x.shape[0]))


def read_paths_file(filename, npart, nslice, bfactor=1):
    """A restart file read as PathReader does (src/algorithm/PathReader.cc:20-140)."""
    out = np.zeros((nslice, npart, 3))
    _check(lib().pimc_paths_read_file(os.fsencode(filename), _dp(out), npart, nslice, bfactor))
    return out


class _Checkpoint:
    """Restart files and random-stream state of one replica (a slot on a server)."""

    def write_paths(self, replica, filename):
        _check(lib().pimc_write_paths(self.h, replica, os.fsencode(filename)))

    def replica_state(self, replica):
        st = ReplicaState()
        _check(lib().pimc_get_replica_state(self.h, replica, C.byref(st)))
        return st.as_dict()

    def set_replica_state(self, replica, state):
        st = ReplicaState.from_dict(state)
        _check(lib().pimc_set_replica_state(self.h, replica, C.byref(st)))


def pair_tables_struct(tables):
    """Array of PairTable from dicts with species/ngpts/norder/rgridinv/logrratioinv/ugrid."""
    n = len(tables)
    arr = (PairTable * max(n, 1))()
    keep = []
    for k, t in enumerate(tables):
        ug = np.ascontiguousarray(t["ugrid"], np.float64)
        keep.append(ug)
        s1, s2 = t["species"]
        arr[k].species1, arr[k].species2 = int(s1), int(s2)
        arr[k].ngpts, arr[k].norder = int(t["ngpts"]), int(t["norder"])
        arr[k].rgridinv, arr[k].logrratioinv = float(t["rgridinv"]), float(t["logrratioinv"])
        arr[k].ugrid = _dp(ug)
    return arr, keep


def ewald_struct(ew):
    if ew is None:
        return None, []
    kv = np.ascontiguousarray(ew["kvec"], np.int32)
    vk = np.ascontiguousarray(ew["vk"], np.float64)
    e = EwaldTable()
    e.totk = int(ew["totk"])
    e.kvec = kv.ctypes.data_as(C.POINTER(C.c_int))
    e.vk = _dp(vk)
    e.one_over_2v = float(ew["one_over_2v"])
    e.self_energy = float(ew["self_energy"])
    for d in range(3):
        e.ikmax[d] = int(ew["ikmax"][d])
    return e, [kv, vk]


def records_to_numpy(recs, n):
    out = {
        "ifirst1": np.array([r.ifirst1 for r in recs[:n]], np.int32),
        "ifirst2": np.array([r.ifirst2 for r in recs[:n]], np.int32),
        "ipart": np.array([r.ipart for r in recs[:n]], np.int32),
        "reject_level": np.array([r.reject_level for r in recs[:n]], np.int32),
        "ds": np.array([list(r.ds) for r in recs[:n]]),
        "ds_node": np.array([list(r.ds_node) for r in recs[:n]]),
        "lnt": np.array([list(r.lnt) for r in recs[:n]]),
    }
    return out


def fp64_peak_tflops():
    """Measured dense FP64 FMA throughput of the device (TFLOP/s)."""
    v = C.c_double()
    _check(lib().pimc_fp64_peak(C.byref(v)))
    return v.value


def fp32_peak_tflops():
    """Measured dense FP32 FMA throughput of the device (TFLOP/s)."""
    v = C.c_double()
    _check(lib().pimc_fp32_peak(C.byref(v)))
    return v.value


def stream_sample(seed, replica, attempt, n):
    """The first n uniforms and normals of one attempt's streams, generated on
    the GPU (for bit-exact comparison with a CPU replay)."""
    u = np.zeros(n)
    z = np.zeros(n)
    _check(lib().pimc_stream_sample(C.c_uint64(seed), replica, attempt, n, _dp(u), _dp(z)))
    return u, z


class Engine(_Checkpoint):
    """A set of replicas advanced on the GPU (pimc_engine).

    ``Engine(system_kw, nreplica, tables, ewald, seed)`` builds replicas of one
    system; ``Engine.batch([kw...], [tables...], seed)`` builds uneven replicas.
    """

    def __init__(self, system_kw=None, nreplica=1, tables=(), ewald=None, seed=20261203,
                 precision=PIMC_PREC_FP64, _handle=None, _systems=None):
        L = lib()
        self.precision = precision
        if _handle is not None:
            self.h = _handle
            self.systems = _systems
        else:
            sysc = system_from_kw(system_kw)
            tabs, self._keep = pair_tables_struct(tables)
            ew, keep2 = ewald_struct(ewald)
            self._keep += keep2
            h = C.c_void_p()
            _check(L.pimc_engine_create(C.byref(sysc), nreplica, tabs, len(tables),
                                        C.byref(ew) if ew is not None else None,
                                        C.c_uint64(seed), precision, C.byref(h)))
            self.h = h
            self.systems = [sysc] * nreplica
        self.nreplica = len(self.systems)
        offs = (C.c_int64 * (self.nreplica + 1))()
        _check(L.pimc_path_offsets(self.h, offs))
        self.offsets = np.array(list(offs), np.int64)

    @classmethod
    def batch(cls, system_kws, tables_per_replica, seed=20261203, precision=PIMC_PREC_FP64):
        L = lib()
        n = len(system_kws)
        systems = (System * n)(*[system_from_kw(kw) for kw in system_kws])
        flat = [t for ts in tables_per_replica for t in ts]
        tabs, keep = pair_tables_struct(flat)
        off = np.zeros(n + 1, np.int32)
        off[1:] = np.cumsum([len(ts) for ts in tables_per_replica])
        h = C.c_void_p()
        _check(L.pimc_engine_create_batch(systems, n, tabs,
                                          off.ctypes.data_as(C.POINTER(C.c_int)),
                                          C.c_uint64(seed), precision, C.byref(h)))
        e = cls(_handle=h, _systems=list(systems), precision=precision)
        e._keep = keep
        return e

    def close(self):
        if getattr(self, "h", None):
            lib().pimc_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        _check(lib().pimc_set_stream(self.h, C.c_void_p(stream_ptr)))

    # paths ----------------------------------------------------------------
    def path_shape(self, r):
        s = self.systems[r]
        return (s.nslice, s.npart, 3)

    def upload_paths(self, paths):
        """paths: one array [nslice][npart][3] per replica, or a packed flat array."""
        if isinstance(paths, np.ndarray) and paths.ndim == 1:
            flat = np.ascontiguousarray(paths, np.float64)
        else:
            flat = np.concatenate([np.ascontiguousarray(p, np.float64).ravel() for p in paths])
        assert flat.size == self.offsets[-1]
        _check(lib().pimc_upload_paths(self.h, _dp(flat)))
        self._last_upload = flat

    def download_paths(self, flat=False, out=None):
        """All replicas' paths; out (a flat float64 array, e.g. a pinned host
        buffer's view) receives them when given."""
        if out is None:
            out = np.empty(int(self.offsets[-1]))
        assert out.dtype == np.float64 and out.size == self.offsets[-1] and out.flags.c_contiguous
        _check(lib().pimc_download_paths(self.h, _dp(out)))
        if flat:
            return out
        return [out[self.offsets[r]:self.offsets[r + 1]].reshape(self.path_shape(r))
                for r in range(self.nreplica)]

    def read_paths(self, replica, filename, bfactor=1):
        """Replaces one replica's path with a restart file's."""
        _check(lib().pimc_read_paths(self.h, replica, os.fsencode(filename), bfactor))

    # sampler --------------------------------------------------------------
    def run_sections(self, nattempt, records=False):
        """nattempt section-move attempts on every replica (asynchronous unless
        records are requested)."""
        if records:
            recs = (MoveRecord * (self.nreplica * nattempt))()
            _check(lib().pimc_run_sections(self.h, nattempt, recs))
            r = records_to_numpy(recs, self.nreplica * nattempt)
            return {k: v.reshape((self.nreplica, nattempt) + v.shape[1:]) for k, v in r.items()}
        _check(lib().pimc_run_sections(self.h, nattempt, None))
        return None

    def run_steps(self, nattempt, nsteps=1, energies=True):
        """nsteps x (nattempt attempts + one energy measurement) as one CUDA
        graph; returns energies [nsteps][nreplica] (or None, asynchronous)."""
        if energies:
            out = np.empty((nsteps, self.nreplica))
            _check(lib().pimc_run_steps(self.h, nattempt, nsteps, _dp(out)))
            return out
        _check(lib().pimc_run_steps(self.h, nattempt, nsteps, None))
        return None

    # launch configuration --------------------------------------------------
    def autotune(self, nattempt=16):
        """Times the candidate launch configurations on nattempt attempts per
        replica (the chains are restored), applies the fastest; returns it and
        every candidate with its time (ms < 0: does not fit)."""
        best = LaunchConfig()
        tried = (LaunchConfig * 32)()
        nt = C.c_int(0)
        _check(lib().pimc_engine_autotune(self.h, nattempt, C.byref(best), tried, 32,
                                          C.byref(nt)))
        return best.as_dict(), [tried[i].as_dict() for i in range(min(nt.value, 32))]

    def configure(self, block, scratch_global=0, ctas_per_sm=0, regs_variant=2):
        cfg = LaunchConfig(block, scratch_global, ctas_per_sm, regs_variant, 0.0)
        _check(lib().pimc_engine_configure(self.h, C.byref(cfg)))

    def launch_config(self):
        cfg = LaunchConfig()
        _check(lib().pimc_engine_get_config(self.h, C.byref(cfg)))
        return cfg.as_dict()

    def run_displace(self, nattempt, box, nmoving=1, species=-1, records=False):
        """nattempt rigid-displacement attempts per replica (uniform box[3])."""
        b = np.ascontiguousarray(box, np.float64)
        if records:
            n = self.nreplica * nattempt
            recs = (DisplaceRecord * max(n, 1))()
            _check(lib().pimc_run_displace(self.h, nattempt, _dp(b), nmoving, species, recs))
            out = {
                "ipart": np.array([[recs[i].ipart[k] for k in range(nmoving)] for i in range(n)],
                                  np.int32),
                "disp": np.array([[list(recs[i].disp[k]) for k in range(nmoving)]
                                  for i in range(n)]),
                "ds": np.array([recs[i].ds for i in range(n)]),
                "ds_node": np.array([recs[i].ds_node for i in range(n)]),
                "accepted": np.array([recs[i].accepted for i in range(n)], np.int32),
            }
            return {k: v.reshape((self.nreplica, nattempt) + v.shape[1:]) for k, v in out.items()}
        _check(lib().pimc_run_displace(self.h, nattempt, _dp(b), nmoving, species, None))
        return None

    def replica_status(self):
        n = self.nreplica
        acc = np.zeros(n, np.int64)
        att = np.zeros(n, np.int64)
        st = np.zeros(n, np.uint32)
        _check(lib().pimc_replica_status(self.h, acc.ctypes.data_as(C.POINTER(C.c_int64)),
                                         att.ctypes.data_as(C.POINTER(C.c_int64)),
                                         st.ctypes.data_as(C.POINTER(C.c_uint32))))
        return acc, att, st

    def node_scale(self, replica, ispec):
        v = C.c_double()
        _check(lib().pimc_node_scale(self.h, replica, ispec, C.byref(v)))
        return v.value

    # estimators -----------------------------------------------------------
    def thermo_energy(self):
        out = np.zeros(self.nreplica)
        _check(lib().pimc_thermo_energy(self.h, _dp(out)))
        return out

    def virial_energy(self, nwindow=1):
        out = np.zeros(self.nreplica)
        _check(lib().pimc_virial_energy(self.h, nwindow, _dp(out)))
        return out

    def coulomb_energy(self, epsilon=1.0):
        out = np.zeros(self.nreplica)
        _check(lib().pimc_coulomb_energy(self.h, epsilon, _dp(out)))
        return out

    def ewald_coulomb_energy(self, epsilon, rcut, est_ewald, vgrid):
        """The optimized-Ewald Coulomb estimator with its own table (dict as
        returned by ewald_estimator_tables) and 1001-point grid."""
        ew, keep = ewald_struct(est_ewald)
        vg = np.ascontiguousarray(vgrid, np.float64)
        out = np.zeros(self.nreplica)
        _check(lib().pimc_ewald_coulomb_energy(self.h, epsilon, rcut, C.byref(ew), _dp(vg),
                                               _dp(out)))
        return out

    # Action / NodeModel level ---------------------------------------------
    def action_difference(self, level, sections, movings, iparts):
        sections = np.ascontiguousarray(sections, np.float64)
        movings = np.ascontiguousarray(movings, np.float64)
        ip = np.ascontiguousarray(iparts, np.int32)
        nb = len(ip)
        ds = np.zeros(nb)
        _check(lib().pimc_action_difference(self.h, level, nb, _dp(sections), _dp(movings),
                                            ip.ctypes.data_as(C.POINTER(C.c_int)), _dp(ds)))
        return ds

    def node_evaluate(self, ispec, r1, r2):
        r1 = np.ascontiguousarray(r1, np.float64)
        r2 = np.ascontiguousarray(r2, np.float64)
        nb, np_ = r1.shape[0], r1.shape[1]
        det = np.zeros(nb)
        d1 = np.zeros((nb, np_))
        d2 = np.zeros((nb, np_))
        err = np.zeros(nb, np.int32)
        _check(lib().pimc_node_evaluate(self.h, ispec, nb, _dp(r1), _dp(r2), _dp(det), _dp(d1),
                                        _dp(d2), err.ctypes.data_as(C.POINTER(C.c_int))))
        return err, det, d1, d2

    @property
    def kernel_launches(self):
        return lib().pimc_kernel_launches(self.h)


class Server(_Checkpoint):
    """Slots of independent simulations over one device pool (pimc_server_*).

    ``admit`` places a simulation in a free slot when its path and Slater-result
    cache fit the pool (returns None when they do not), ``run`` advances every
    admitted slot in one persistent launch, ``release`` frees the slot and its
    memory.  Each simulation draws the random stream of its own ``stream_id``.
    """

    def __init__(self, slots, hbm_bytes, max_npart, max_nslice, max_level, max_node_count,
                 seed=20261203, precision=PIMC_PREC_FP64):
        L = lib()
        cfg = ServerConfig(slots, hbm_bytes, max_npart, max_nslice, max_level, max_node_count)
        h = C.c_void_p()
        _check(L.pimc_server_create(C.byref(cfg), C.c_uint64(seed), precision, C.byref(h)))
        self.h = h
        self.slots = slots
        self.systems = [None] * slots
        self._keep = [None] * slots

    def close(self):
        if getattr(self, "h", None):
            lib().pimc_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def configure(self, block=256, scratch_global=0, regs_variant=2):
        """Launch shape of every round (before the first admission)."""
        cfg = LaunchConfig(block, scratch_global, 0, regs_variant, 0.0)
        _check(lib().pimc_engine_configure(self.h, C.byref(cfg)))

    def set_stream(self, stream_ptr):
        _check(lib().pimc_set_stream(self.h, C.c_void_p(stream_ptr)))

    def admit(self, system_kw, tables, path, stream_id, round_attempts):
        sysc = system_from_kw(system_kw)
        tabs, keep = pair_tables_struct(tables)
        flat = np.ascontiguousarray(path, np.float64).ravel()
        assert flat.size == 3 * sysc.nslice * sysc.npart
        slot = C.c_int(-1)
        rc = lib().pimc_server_admit(self.h, C.byref(sysc), tabs, len(tables), _dp(flat),
                                     C.c_uint32(stream_id), int(round_attempts), C.byref(slot))
        if rc == PIMC_ERR_CAPACITY:
            return None
        _check(rc)
        self.systems[slot.value] = sysc
        self._keep[slot.value] = (keep, tables)
        return slot.value

    def release(self, slot):
        _check(lib().pimc_server_release(self.h, slot))
        self.systems[slot] = None
        self._keep[slot] = None

    def run(self):
        """One round: every slot advances its own round_attempts."""
        _check(lib().pimc_server_run(self.h))

    def energies(self, slots=None):
        """Thermodynamic energy of every slot (NaN for free slots), or of the
        listed active slots only (in that order)."""
        if slots is None:
            out = np.empty(self.slots)
            _check(lib().pimc_server_energy(self.h, _dp(out)))
            return out
        idx = np.ascontiguousarray(slots, np.int32)
        out = np.empty(len(idx))
        if len(idx):
            _check(lib().pimc_server_energy_slots(self.h, idx.ctypes.data_as(C.POINTER(C.c_int)),
                                                  len(idx), _dp(out)))
        return out

    def download_path(self, slot):
        s = self.systems[slot]
        out = np.empty((s.nslice, s.npart, 3))
        _check(lib().pimc_server_download_path(self.h, slot, _dp(out)))
        return out

    def pool(self):
        used, big = C.c_size_t(), C.c_size_t()
        _check(lib().pimc_server_pool(self.h, C.byref(used), C.byref(big)))
        return used.value, big.value

    def replica_status(self):
        n = self.slots
        acc = np.zeros(n, np.int64)
        att = np.zeros(n, np.int64)
        st = np.zeros(n, np.uint32)
        _check(lib().pimc_replica_status(self.h, acc.ctypes.data_as(C.POINTER(C.c_int64)),
                                         att.ctypes.data_as(C.POINTER(C.c_int64)),
                                         st.ctypes.data_as(C.POINTER(C.c_uint32))))
        return acc, att, st

    def kernel_launches(self):
        return lib().pimc_kernel_launches(self.h)


def coulomb_tables(system_kw, norder=3, ngpts=0, rmin=0.0, rmax=0.0, ewald_rcut=0.0):
    """CoulombAction pair tables (and the OptEwaldSum table when the system has
    Ewald) built by the engine's own host code; returns (tables, ewald) in the
    form Engine() takes."""
    L = lib()
    if not hasattr(L, "_tables_bound"):
        L.pimc_coulomb_tables.argtypes = [C.POINTER(System), C.c_int, C.c_int, C.c_double,
                                          C.c_double, C.c_double, C.c_double,
                                          C.POINTER(C.POINTER(PairTable)), C.POINTER(C.c_int),
                                          C.POINTER(C.POINTER(EwaldTable))]
        L._tables_bound = True
    s = system_from_kw(system_kw)
    tp = C.POINTER(PairTable)()
    nt = C.c_int()
    ep = C.POINTER(EwaldTable)()
    _check(L.pimc_coulomb_tables(C.byref(s), norder, ngpts, rmin, rmax, ewald_rcut,
                                 float(system_kw.get("ewald_kcut", 0.0)), C.byref(tp),
                                 C.byref(nt), C.byref(ep)))
    tables = []
    for k in range(nt.value):
        t = tp[k]
        nd = t.norder + 1
        ug = np.ctypeslib.as_array(t.ugrid, shape=(t.ngpts * 2 * nd,)).reshape(t.ngpts, 2, nd).copy()
        tables.append(dict(species=(t.species1, t.species2), ngpts=t.ngpts, norder=t.norder,
                           rgridinv=t.rgridinv, logrratioinv=t.logrratioinv, ugrid=ug))
    ewald = None
    if ep:
        e = ep.contents
        ewald = dict(totk=e.totk,
                     kvec=np.ctypeslib.as_array(e.kvec, shape=(e.totk * 3,)).reshape(-1, 3).copy(),
                     vk=np.ctypeslib.as_array(e.vk, shape=(e.totk,)).copy(),
                     one_over_2v=e.one_over_2v, self_energy=e.self_energy, ikmax=list(e.ikmax))
    return tables, ewald


def ewald_estimator_tables(system_kw, rcut, kcut, epsilon=1.0):
    """The optimized Ewald sum an EwaldCoulombEstimator builds for itself: its
    k-list table (dict) and the 1001-point grid -f(i rcut/1000)/epsilon."""
    L = lib()
    s = system_from_kw(system_kw)
    ep = C.POINTER(EwaldTable)()
    vg = np.zeros(1001)
    _check(L.pimc_ewald_estimator_tables(C.byref(s), rcut, kcut, epsilon, C.byref(ep), _dp(vg)))
    e = ep.contents
    ew = dict(totk=e.totk,
              kvec=np.ctypeslib.as_array(e.kvec, shape=(e.totk * 3,)).reshape(-1, 3).copy(),
              vk=np.ctypeslib.as_array(e.vk, shape=(e.totk,)).copy(),
              one_over_2v=e.one_over_2v, self_energy=e.self_energy, ikmax=list(e.ikmax))
    return ew, vg
