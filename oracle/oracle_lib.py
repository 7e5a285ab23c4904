"""ctypes bindings for the two CPU checkers (test infrastructure only).

``RefOracle`` drives pi-qmc's own hot-path objects (oracle/_ref/libpimcref.so,
built from the reference tree where it exists).  ``PortOracle`` drives the C++
restatement (oracle/liboracle_port.so, built on every machine by
``build_port()``).  Both take the same ``ora_config`` and return the same
records, so tests can hold one against the other and against the engine.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PORT_LIB = os.path.join(HERE, "liboracle_port.so")
REF_LIB = os.path.join(HERE, "_ref", "libpimcref.so")
MAXS = 4
MAXL = 8


class OraConfig(C.Structure):
    _fields_ = [
        ("npart", C.c_int), ("nspecies", C.c_int),
        ("spec_count", C.c_int * MAXS), ("spec_mass", C.c_double * MAXS),
        ("spec_charge", C.c_double * MAXS), ("sho_omega", C.c_double * MAXS),
        ("prim_a", C.c_double * MAXS), ("prim_b", C.c_double * MAXS),
        ("node_kind", C.c_int * MAXS), ("node_omega", C.c_double * MAXS),
        ("node_temperature", C.c_double), ("nslice", C.c_int), ("tau", C.c_double),
        ("temperature", C.c_double), ("nlevel", C.c_int), ("cell", C.c_double * 3),
        ("spring", C.c_int), ("coulomb", C.c_int), ("epsilon", C.c_double),
        ("norder", C.c_int), ("ngpts", C.c_int), ("ewald", C.c_int),
        ("ewald_rcut", C.c_double), ("ewald_kcut", C.c_double), ("mover", C.c_int),
        ("seed", C.c_uint64), ("replica", C.c_uint32),
        ("delayed_rejection", C.c_int), ("sigma_factor", C.c_double),
        ("dr_sigma_factor", C.c_double),
    ]


class OraRecord(C.Structure):
    _fields_ = [
        ("ifirst1", C.c_int), ("ifirst2", C.c_int), ("ipart", C.c_int),
        ("reject_level", C.c_int), ("ds", C.c_double * (MAXL + 1)),
        ("ds_node", C.c_double * (MAXL + 1)), ("lnt", C.c_double * (MAXL + 1)),
    ]


MAXMOV = 4


class OraDRecord(C.Structure):
    _fields_ = [("ipart", C.c_int * MAXMOV), ("disp", (C.c_double * 3) * MAXMOV),
                ("ds", C.c_double), ("ds_node", C.c_double), ("accepted", C.c_int)]


def drecords_to_numpy(recs, n, nmoving):
    return {
        "ipart": np.array([[recs[i].ipart[k] for k in range(nmoving)] for i in range(n)],
                          np.int32),
        "disp": np.array([[list(recs[i].disp[k]) for k in range(nmoving)] for i in range(n)]),
        "ds": np.array([recs[i].ds for i in range(n)]),
        "ds_node": np.array([recs[i].ds_node for i in range(n)]),
        "accepted": np.array([recs[i].accepted for i in range(n)], np.int32),
    }


class OraPairTable(C.Structure):
    _fields_ = [("ngpts", C.c_int), ("norder", C.c_int), ("rgridinv", C.c_double),
                ("logrratioinv", C.c_double), ("ugrid", C.POINTER(C.c_double))]


class OraEwaldTable(C.Structure):
    _fields_ = [("totk", C.c_int), ("kvec", C.POINTER(C.c_int)),
                ("vk", C.POINTER(C.c_double)), ("one_over_2v", C.c_double),
                ("self_energy", C.c_double), ("ikmax", C.c_int * 3)]


def make_config(**kw):
    """Build an OraConfig from keyword arguments (species given as lists)."""
    c = OraConfig()
    counts = kw["counts"]
    c.nspecies = len(counts)
    c.npart = int(sum(counts))
    for i, n in enumerate(counts):
        c.spec_count[i] = n
        c.spec_mass[i] = kw.get("masses", [1.0] * len(counts))[i]
        c.spec_charge[i] = kw.get("charges", [-1.0] * len(counts))[i]
        c.sho_omega[i] = kw.get("sho_omega", [0.0] * len(counts))[i]
        c.prim_a[i] = kw.get("prim_a", [0.0] * len(counts))[i]
        c.prim_b[i] = kw.get("prim_b", [0.0] * len(counts))[i]
        c.node_kind[i] = kw.get("node_kind", [0] * len(counts))[i]
        c.node_omega[i] = kw.get("node_omega", [0.0] * len(counts))[i]
    c.nslice = kw["nslice"]
    c.tau = kw["beta"] / kw["nslice"]
    c.temperature = 1.0 / kw["beta"]
    c.node_temperature = kw.get("node_temperature", c.temperature)
    c.nlevel = kw["nlevel"]
    cell = kw.get("cell", 1000.0)
    for d in range(3):
        c.cell[d] = cell
    c.spring = kw.get("spring", 1)
    c.coulomb = kw.get("coulomb", 0)
    c.epsilon = kw.get("epsilon", 1.0)
    c.norder = kw.get("norder", 3)
    c.ngpts = kw.get("ngpts", 0)
    c.ewald = kw.get("ewald", 0)
    c.ewald_rcut = kw.get("ewald_rcut", 0.0)
    c.ewald_kcut = kw.get("ewald_kcut", 0.0)
    c.mover = kw.get("mover", 0)
    c.seed = kw.get("seed", 20261203)
    c.replica = kw.get("replica", 0)
    c.delayed_rejection = int(kw.get("delayed_rejection", 0))
    c.sigma_factor = kw.get("sigma_factor", 0.0)
    c.dr_sigma_factor = kw.get("dr_sigma_factor", 0.0)
    return c


def build_port(force=False):
    """Compile the restatement (plain g++, no reference headers needed)."""
    src = os.path.join(HERE, "port.cc")
    if (not force and os.path.exists(PORT_LIB)
            and os.path.getmtime(PORT_LIB) >= max(
                os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "oracle_api.h")),
                os.path.getmtime(os.path.join(REPO, "pi-qmc_gb300", "csrc", "pimc_rng.h")))):
        return PORT_LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", PORT_LIB, src]
    subprocess.run(cmd, check=True)
    return PORT_LIB


def cpu_stream(seed, replica, attempt, n):
    """Uniforms and normals of one attempt's streams, computed on the CPU."""
    L = PortOracle.lib()
    L.port_stream_sample.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_int,
                                     C.POINTER(C.c_double), C.POINTER(C.c_double)]
    u = np.zeros(n)
    z = np.zeros(n)
    L.port_stream_sample(C.c_uint64(seed), replica, attempt, n, _dp(u), _dp(z))
    return u, z


def records_to_numpy(recs, n):
    out = {
        "ifirst1": np.array([recs[i].ifirst1 for i in range(n)], np.int32),
        "ifirst2": np.array([recs[i].ifirst2 for i in range(n)], np.int32),
        "ipart": np.array([recs[i].ipart for i in range(n)], np.int32),
        "reject_level": np.array([recs[i].reject_level for i in range(n)], np.int32),
        "ds": np.array([list(recs[i].ds) for i in range(n)]),
        "ds_node": np.array([list(recs[i].ds_node) for i in range(n)]),
        "lnt": np.array([list(recs[i].lnt) for i in range(n)]),
    }
    return out


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class _Base:
    def __init__(self, cfg):
        self.cfg = cfg
        self.nsec = (1 << cfg.nlevel) + 1

    def get_path(self):
        out = np.zeros((self.cfg.nslice, self.cfg.npart, 3))
        self._get(self.h, _dp(out))
        return out

    def set_path(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        assert xyz.shape == (self.cfg.nslice, self.cfg.npart, 3)
        self._set(self.h, _dp(xyz))

    def run(self, n, first_attempt=0):
        recs = (OraRecord * max(n, 1))()
        nacc = self._run(self.h, n, first_attempt, recs)
        r = records_to_numpy(recs, n)
        r["naccepted"] = nacc
        return r

    def run_displace(self, n, dist, nmoving=1, species=-1, first_attempt=0):
        """n rigid-displacement attempts (uniform box dist[3]); records per attempt."""
        recs = (OraDRecord * max(n, 1))()
        d = (C.c_double * 3)(*[float(x) for x in dist])
        nacc = self._run_displace(self.h, n, first_attempt, d, nmoving, species, recs)
        r = drecords_to_numpy(recs, n, nmoving)
        r["naccepted"] = nacc
        return r


class RefOracle(_Base):
    """pi-qmc's own code (requires oracle/_ref/libpimcref.so)."""
    _lib = None

    @classmethod
    def available(cls):
        return os.path.exists(REF_LIB)

    @classmethod
    def lib(cls):
        if cls._lib is None:
            L = C.CDLL(REF_LIB)
            L.ref_create.restype = C.c_void_p
            L.ref_create.argtypes = [C.POINTER(OraConfig)]
            for f in ("ref_set_path", "ref_get_path"):
                getattr(L, f).argtypes = [C.c_void_p, C.POINTER(C.c_double)]
            L.ref_run.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.POINTER(OraRecord)]
            L.ref_run_displace.argtypes = [C.c_void_p, C.c_int, C.c_uint32,
                                           C.POINTER(C.c_double), C.c_int, C.c_int,
                                           C.POINTER(OraDRecord)]
            L.ref_thermo_energy.restype = C.c_double
            L.ref_thermo_energy.argtypes = [C.c_void_p]
            L.ref_virial_energy.restype = C.c_double
            L.ref_virial_energy.argtypes = [C.c_void_p, C.c_int]
            L.ref_coulomb_energy.restype = C.c_double
            L.ref_coulomb_energy.argtypes = [C.c_void_p, C.c_double]
            L.ref_estimator_ewald.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double,
                                              C.POINTER(C.c_int), C.POINTER(C.c_int),
                                              C.POINTER(C.c_double), C.POINTER(C.c_double),
                                              C.POINTER(C.c_int), C.POINTER(C.c_double)]
            L.ref_ewald_coulomb_energy.restype = C.c_double
            L.ref_ewald_coulomb_energy.argtypes = [C.c_void_p, C.c_double, C.c_double,
                                                   C.c_double]
            L.ref_bead_action.argtypes = [C.c_void_p, C.c_int, C.c_int,
                                          C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.ref_action_diff.restype = C.c_double
            L.ref_action_diff.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.c_int,
                                          C.POINTER(C.c_int)]
            L.ref_node_eval.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.c_int, C.c_int,
                                        C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]
            L.ref_node_scale.restype = C.c_double
            L.ref_node_scale.argtypes = [C.c_void_p, C.c_int]
            L.ref_set_node_scale.argtypes = [C.c_void_p, C.c_int, C.c_double]
            L.ref_num_pair_tables.argtypes = [C.c_void_p]
            L.ref_pair_table.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int),
                                         C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.ref_ewald.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_int)]
            L.ref_ewald_long_range.restype = C.c_double
            L.ref_ewald_long_range.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
            L.ref_coulomb_u.restype = C.c_double
            L.ref_coulomb_u.argtypes = [C.c_void_p, C.c_double, C.c_int]
            L.ref_coulomb_utau.restype = C.c_double
            L.ref_coulomb_utau.argtypes = [C.c_void_p, C.c_double, C.c_int]
            L.ref_write_paths.argtypes = [C.c_void_p, C.c_char_p]
            L.ref_read_paths.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
            cls._lib = L
        return cls._lib

    def __init__(self, cfg):
        super().__init__(cfg)
        L = self.lib()
        self._cfg_keep = cfg
        self.h = C.c_void_p(L.ref_create(C.byref(cfg)))
        self._get, self._set, self._run = L.ref_get_path, L.ref_set_path, L.ref_run
        self._run_displace = L.ref_run_displace

    def virial_energy(self, nwindow=1):
        return self.lib().ref_virial_energy(self.h, nwindow)

    def coulomb_energy(self, epsilon=1.0):
        return self.lib().ref_coulomb_energy(self.h, epsilon)

    def ewald_coulomb_energy(self, epsilon, rcut, kcut):
        return self.lib().ref_ewald_coulomb_energy(self.h, epsilon, rcut, kcut)

    def estimator_ewald(self, epsilon, rcut, kcut):
        """The estimator's own Ewald table and short-range grid."""
        L = self.lib()
        totk = C.c_int(0)
        scal = (C.c_double * 2)()
        ik = (C.c_int * 3)()
        L.ref_estimator_ewald(self.h, rcut, kcut, epsilon, C.byref(totk), None, None, scal, ik,
                              None)
        n = totk.value
        kv = np.zeros(3 * n, np.int32)
        vk = np.zeros(n)
        vg = np.zeros(1001)
        L.ref_estimator_ewald(self.h, rcut, kcut, epsilon, C.byref(totk),
                              kv.ctypes.data_as(C.POINTER(C.c_int)),
                              vk.ctypes.data_as(C.POINTER(C.c_double)), scal, ik,
                              vg.ctypes.data_as(C.POINTER(C.c_double)))
        return dict(totk=n, kvec=kv.reshape(n, 3), vk=vk, one_over_2v=scal[0],
                    self_energy=scal[1], ikmax=list(ik)), vg

    def thermo_energy(self):
        return self.lib().ref_thermo_energy(self.h)

    def write_paths(self, filename):
        """WritePaths::run on the current path (pi-qmc's restart file)."""
        self.lib().ref_write_paths(self.h, os.fsencode(filename))

    def read_paths(self, filename, bfactor=1):
        """PathReader::run into the current path."""
        self.lib().ref_read_paths(self.h, os.fsencode(filename), bfactor)

    def action_diff(self, level, section, moving, ipart):
        section = np.ascontiguousarray(section, np.float64)
        moving = np.ascontiguousarray(moving, np.float64)
        idx = (C.c_int * 1)(ipart)
        return self.lib().ref_action_diff(self.h, level, _dp(section), _dp(moving), 1, idx)

    def node_eval(self, ispec, r1, r2, islice, scale_magnitude):
        r1 = np.ascontiguousarray(r1, np.float64)
        r2 = np.ascontiguousarray(r2, np.float64)
        det = C.c_double()
        d1 = np.zeros(self.cfg.npart)
        d2 = np.zeros(self.cfg.npart)
        err = self.lib().ref_node_eval(self.h, ispec, _dp(r1), _dp(r2), islice,
                                       int(scale_magnitude), C.byref(det), _dp(d1), _dp(d2))
        return err, det.value, d1, d2

    def node_scale(self, ispec):
        return self.lib().ref_node_scale(self.h, ispec)

    def pair_tables(self):
        """List of dicts (species pair, grid parameters, ugrid) in construction order."""
        L = self.lib()
        out = []
        for k in range(L.ref_num_pair_tables(self.h)):
            info = (C.c_int * 8)()
            gp = (C.c_double * 3)()
            L.ref_pair_table(self.h, k, info, gp, None)
            ng, norder, ndata = info[0], info[1], info[6]
            ug = np.zeros((ng, 2, ndata))
            L.ref_pair_table(self.h, k, info, gp, _dp(ug))
            out.append(dict(ngpts=ng, norder=norder, ifirst1=info[2], npart1=info[3],
                            ifirst2=info[4], npart2=info[5], exlevel=info[7],
                            rgridinv=gp[0], logrratioinv=gp[1], mass=gp[2], ugrid=ug))
        return out

    def ewald_table(self):
        L = self.lib()
        totk = C.c_int()
        scal = np.zeros(16)
        ik = (C.c_int * 3)()
        if L.ref_ewald(self.h, C.byref(totk), None, None, _dp(scal), ik) != 0:
            return None
        kv = np.zeros((totk.value, 3), np.int32)
        vk = np.zeros(totk.value)
        L.ref_ewald(self.h, C.byref(totk), kv.ctypes.data_as(C.POINTER(C.c_int)), _dp(vk),
                    _dp(scal), ik)
        return dict(totk=totk.value, kvec=kv, vk=vk, one_over_2v=scal[0],
                    self_energy=scal[1], coef=scal[2:10].copy(), ikmax=list(ik))

    def ewald_long_range(self, r):
        r = np.ascontiguousarray(r, np.float64)
        return self.lib().ref_ewald_long_range(self.h, _dp(r))


def species_pair_of(tab, cfg):
    """Map a table's (ifirst, npart) pairs back to species indices."""
    firsts = np.cumsum([0] + [cfg.spec_count[i] for i in range(cfg.nspecies)])[:-1]
    s1 = int(np.nonzero(firsts == tab["ifirst1"])[0][0])
    s2 = int(np.nonzero(firsts == tab["ifirst2"])[0][0])
    return s1, s2


class PortOracle(_Base):
    """The C++ restatement; takes pair/Ewald tables as inputs."""
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            build_port()
            L = C.CDLL(PORT_LIB)
            L.port_create.restype = C.c_void_p
            L.port_create.argtypes = [C.POINTER(OraConfig), C.c_int, C.POINTER(C.c_int),
                                      C.POINTER(OraPairTable), C.POINTER(OraEwaldTable)]
            L.port_destroy.argtypes = [C.c_void_p]
            for f in ("port_set_path", "port_get_path"):
                getattr(L, f).argtypes = [C.c_void_p, C.POINTER(C.c_double)]
            L.port_run.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.POINTER(OraRecord)]
            L.port_thermo_energy.restype = C.c_double
            L.port_thermo_energy.argtypes = [C.c_void_p]
            L.port_bead_utau.restype = C.c_double
            L.port_bead_utau.argtypes = [C.c_void_p, C.c_int, C.c_int]
            L.port_action_diff.restype = C.c_double
            L.port_action_diff.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                           C.POINTER(C.c_double), C.c_int]
            L.port_node_eval.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.c_int, C.c_int,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]
            L.port_node_scale.restype = C.c_double
            L.port_node_scale.argtypes = [C.c_void_p, C.c_int]
            L.port_set_node_scale.argtypes = [C.c_void_p, C.c_int, C.c_double]
            L.port_init_errors.argtypes = [C.c_void_p]
            L.port_ewald_long_range.restype = C.c_double
            L.port_ewald_long_range.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
            L.port_run_displace.argtypes = [C.c_void_p, C.c_int, C.c_uint32,
                                            C.POINTER(C.c_double), C.c_int, C.c_int,
                                            C.POINTER(OraDRecord)]
            L.port_virial_energy.restype = C.c_double
            L.port_virial_energy.argtypes = [C.c_void_p, C.c_int]
            L.port_coulomb_energy.restype = C.c_double
            L.port_coulomb_energy.argtypes = [C.c_void_p, C.c_double]
            L.port_ewald_coulomb_energy.restype = C.c_double
            L.port_ewald_coulomb_energy.argtypes = [C.c_void_p, C.c_double, C.c_double,
                                                    C.POINTER(OraEwaldTable),
                                                    C.POINTER(C.c_double)]
            cls._lib = L
        return cls._lib

    def __init__(self, cfg, pair_tables=(), ewald=None):
        super().__init__(cfg)
        L = self.lib()
        n = len(pair_tables)
        self._keep = []
        tabs = (OraPairTable * max(n, 1))()
        sp = (C.c_int * max(2 * n, 2))()
        for k, t in enumerate(pair_tables):
            ug = np.ascontiguousarray(t["ugrid"], np.float64)
            self._keep.append(ug)
            tabs[k].ngpts = t["ngpts"]
            tabs[k].norder = t["norder"]
            tabs[k].rgridinv = t["rgridinv"]
            tabs[k].logrratioinv = t["logrratioinv"]
            tabs[k].ugrid = _dp(ug)
            s1, s2 = t["species"] if "species" in t else species_pair_of(t, cfg)
            sp[2 * k], sp[2 * k + 1] = s1, s2
        ew = None
        if ewald is not None:
            kv = np.ascontiguousarray(ewald["kvec"], np.int32)
            vk = np.ascontiguousarray(ewald["vk"], np.float64)
            self._keep += [kv, vk]
            ew = OraEwaldTable()
            ew.totk = int(ewald["totk"])
            ew.kvec = kv.ctypes.data_as(C.POINTER(C.c_int))
            ew.vk = _dp(vk)
            ew.one_over_2v = float(ewald["one_over_2v"])
            ew.self_energy = float(ewald["self_energy"])
            for d in range(3):
                ew.ikmax[d] = int(ewald["ikmax"][d])
        self._cfg_keep = cfg
        self.h = C.c_void_p(L.port_create(C.byref(cfg), n, sp, tabs,
                                          C.byref(ew) if ew is not None else None))
        self._get, self._set, self._run = L.port_get_path, L.port_set_path, L.port_run
        self._run_displace = L.port_run_displace

    def __del__(self):
        try:
            self.lib().port_destroy(self.h)
        except Exception:
            pass

    def virial_energy(self, nwindow=1):
        return self.lib().port_virial_energy(self.h, nwindow)

    def coulomb_energy(self, epsilon=1.0):
        return self.lib().port_coulomb_energy(self.h, epsilon)

    def ewald_coulomb_energy(self, epsilon, rcut, est_ewald, vgrid):
        """est_ewald: dict(totk, kvec, vk, one_over_2v, self_energy, ikmax) of the
        estimator's own Ewald sum; vgrid: its 1001-point -evalFR/epsilon grid."""
        kv = np.ascontiguousarray(est_ewald["kvec"], np.int32).ravel()
        vk = np.ascontiguousarray(est_ewald["vk"], np.float64)
        vg = np.ascontiguousarray(vgrid, np.float64)
        et = OraEwaldTable()
        et.totk = int(est_ewald["totk"])
        et.kvec = kv.ctypes.data_as(C.POINTER(C.c_int))
        et.vk = vk.ctypes.data_as(C.POINTER(C.c_double))
        et.one_over_2v = float(est_ewald["one_over_2v"])
        et.self_energy = float(est_ewald["self_energy"])
        for d in range(3):
            et.ikmax[d] = int(est_ewald["ikmax"][d])
        return self.lib().port_ewald_coulomb_energy(self.h, epsilon, rcut, C.byref(et),
                                                    vg.ctypes.data_as(C.POINTER(C.c_double)))

    def thermo_energy(self):
        return self.lib().port_thermo_energy(self.h)

    def action_diff(self, level, section, moving, ipart):
        section = np.ascontiguousarray(section, np.float64)
        moving = np.ascontiguousarray(moving, np.float64)
        return self.lib().port_action_diff(self.h, level, _dp(section), _dp(moving), ipart)

    def node_eval(self, ispec, r1, r2, islice, scale_magnitude):
        r1 = np.ascontiguousarray(r1, np.float64)
        r2 = np.ascontiguousarray(r2, np.float64)
        det = C.c_double()
        d1 = np.zeros(self.cfg.npart)
        d2 = np.zeros(self.cfg.npart)
        err = self.lib().port_node_eval(self.h, ispec, _dp(r1), _dp(r2), islice,
                                        int(scale_magnitude), C.byref(det), _dp(d1), _dp(d2))
        return err, det.value, d1, d2

    def node_scale(self, ispec):
        return self.lib().port_node_scale(self.h, ispec)

    def ewald_long_range(self, r):
        r = np.ascontiguousarray(r, np.float64)
        return self.lib().port_ewald_long_range(self.h, _dp(r))
