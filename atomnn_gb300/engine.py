"""Python binding of the C ABI in include/nnpgpu.h (libnnpgpu.so, built in-tree).

The engine runs only on the GPU: loading fails loudly when the shared library is missing, and
context creation fails when no CUDA device is present.  There is no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libnnpgpu.so")

OK, ERR_INVALID, ERR_IO, ERR_CUDA, ERR_OOM, ERR_CAPACITY, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_BUSY = 0, -1, -2, -3, -4, -5, -6, -7, -8
ENERGY, FORCE, SYMM, BF16, NO_VACUUM, BATCHED = 0x1, 0x2, 0x4, 0x8, 0x10, 0x20

# every symbol the header declares
EXPORTS = ["nnpgpu_create", "nnpgpu_destroy", "nnpgpu_last_error", "nnpgpu_ntypes", "nnpgpu_type_index", "nnpgpu_cutoff",
           "nnpgpu_ninput", "nnpgpu_compute", "nnpgpu_compute_device", "nnpgpu_neighbors", "nnpgpu_neighbors_rc", "nnpgpu_serve_start", "nnpgpu_submit",
           "nnpgpu_poll", "nnpgpu_serve_stop", "nnpgpu_profile_enable", "nnpgpu_profile_read",
           "nnpgpu_profile_stage_name", "nnpgpu_symm_noalloc", "nnpgpu_autotune", "nnpgpu_get_tune", "nnpgpu_set_tune", "nnpgpu_set_wait_limit", "nnpgpu_md_create", "nnpgpu_md_forces", "nnpgpu_md_run",
           "nnpgpu_md_state", "nnpgpu_md_destroy", "nnpgpu_nparams", "nnpgpu_train_grad", "nnpgpu_energy_symm",
           "nnpgpu_train_force_grad", "nnpgpu_get_params", "nnpgpu_set_params", "nnpgpu_write_potential"]

_lib = None


class NNPGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("nnpgpu error %d: %s" % (code, msg))
        self.code = code


class Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("max_neighbors", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_size_t),
                ("verbose", ctypes.c_int)]


class ServeOpts(ctypes.Structure):
    _fields_ = [("max_batch_atoms", ctypes.c_int), ("max_inflight", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_size_t),
                ("skin", ctypes.c_double), ("flags", ctypes.c_int)]


def load_library(path=LIB_PATH):
    """Load libnnpgpu.so; raises if it has not been built (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libnnpgpu.so not built (%s): run `python -c 'import __graft_entry__ as g; g.build()'`" % path)
    L = ctypes.CDLL(path)
    vp, ip, dp, cp, szp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_char_p, ctypes.c_size_t
    L.nnpgpu_create.argtypes = [cp, ctypes.POINTER(Opts), ctypes.POINTER(vp)]
    L.nnpgpu_destroy.argtypes = [vp]
    L.nnpgpu_destroy.restype = None
    L.nnpgpu_last_error.argtypes = [vp]
    L.nnpgpu_last_error.restype = cp
    L.nnpgpu_ntypes.argtypes = [vp]
    L.nnpgpu_type_index.argtypes = [vp, cp]
    L.nnpgpu_cutoff.argtypes = [vp]
    L.nnpgpu_cutoff.restype = dp
    L.nnpgpu_ninput.argtypes = [vp, ip]
    L.nnpgpu_compute.argtypes = [vp, ip, vp, vp, vp, vp, ip, vp, vp, vp]
    L.nnpgpu_compute_device.argtypes = [vp, ip, vp, vp, vp, vp, ip, vp, vp, vp, vp]
    L.nnpgpu_neighbors.argtypes = [vp, ip, vp, vp, ip, vp, vp, vp, vp, vp]
    L.nnpgpu_neighbors_rc.argtypes = [vp, dp, ip, vp, vp, ip, vp, vp, vp, vp, vp]
    L.nnpgpu_autotune.argtypes = [vp, ip, vp, vp, vp, vp, ip, ctypes.c_char_p, ip]
    L.nnpgpu_get_tune.argtypes = [vp, vp, vp, vp, vp]
    L.nnpgpu_set_tune.argtypes = [vp, ip, ip, ip, ip]
    L.nnpgpu_set_wait_limit.argtypes = [vp, ip]
    L.nnpgpu_md_create.argtypes = [vp, ip, vp, vp, vp, vp, vp, dp, dp, ip, ctypes.POINTER(vp)]
    L.nnpgpu_md_forces.argtypes = [vp, vp]
    L.nnpgpu_md_run.argtypes = [vp, ip, vp, vp]
    L.nnpgpu_md_state.argtypes = [vp, vp, vp, vp, vp]
    L.nnpgpu_nparams.argtypes = [vp, ip]
    L.nnpgpu_train_grad.argtypes = [vp, ip, vp, vp, vp, vp, vp, ip, dp, vp, vp]
    L.nnpgpu_energy_symm.argtypes = [vp, ip, vp, vp, vp, ip, ip, vp]
    L.nnpgpu_train_force_grad.argtypes = [vp, ip, vp, vp, vp, vp, vp, vp, dp, ip, dp, vp, vp]
    L.nnpgpu_get_params.argtypes = [vp, ip, vp]
    L.nnpgpu_set_params.argtypes = [vp, ip, vp]
    L.nnpgpu_write_potential.argtypes = [vp, cp]
    L.nnpgpu_md_destroy.argtypes = [vp]
    L.nnpgpu_md_destroy.restype = None
    L.nnpgpu_serve_start.argtypes = [vp, ctypes.POINTER(ServeOpts)]
    L.nnpgpu_submit.argtypes = [vp, ip, vp, vp, vp, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]
    L.nnpgpu_poll.argtypes = [vp, ctypes.c_longlong, vp, vp, ctypes.POINTER(ctypes.c_double)]
    L.nnpgpu_serve_stop.argtypes = [vp]
    L.nnpgpu_profile_enable.argtypes = [vp, ip]
    L.nnpgpu_profile_read.argtypes = [vp, ip, ctypes.POINTER(dp), ctypes.POINTER(ctypes.c_longlong)]
    L.nnpgpu_profile_stage_name.argtypes = [ip]
    L.nnpgpu_profile_stage_name.restype = cp
    L.nnpgpu_symm_noalloc.argtypes = [vp, ip, vp, vp, vp, vp, ip, vp]
    _lib = L
    return L


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _cell_colmajor(cell):
    if cell is None:
        return np.zeros(9)
    return np.ascontiguousarray(np.asarray(cell, dtype=np.float64).T).ravel()


class Engine:
    """A context of the GPU engine for one potential file (nnpgpu_create)."""

    def __init__(self, potfile, device=0, max_neighbors=0, hbm_budget_bytes=0):
        self.lib = load_library()
        self._ctx = ctypes.c_void_p()
        o = Opts(device, max_neighbors, hbm_budget_bytes, 0)
        rc = self.lib.nnpgpu_create(potfile.encode(), ctypes.byref(o), ctypes.byref(self._ctx))
        if rc != OK:
            msg = self.lib.nnpgpu_last_error(self._ctx).decode() if self._ctx else ""
            if self._ctx:
                self.lib.nnpgpu_destroy(self._ctx)
                self._ctx = None
            raise NNPGPUError(rc, msg)
        self.ntypes = self.lib.nnpgpu_ntypes(self._ctx)
        self.rc = self.lib.nnpgpu_cutoff(self._ctx)
        self.ninput = [self.lib.nnpgpu_ninput(self._ctx, t) for t in range(self.ntypes)]

    def close(self):
        if getattr(self, "_ctx", None):
            self.lib.nnpgpu_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc != OK:
            raise NNPGPUError(rc, self.lib.nnpgpu_last_error(self._ctx).decode())

    def type_index(self, name):
        return self.lib.nnpgpu_type_index(self._ctx, name.encode())

    def compute(self, structures, flags=ENERGY | FORCE):
        """structures: list of objects with .posn (N,3), .species (N,), .cell (3x3, columns =
        lattice vectors).  Returns (energies [nstruc], forces list [(N,3)] or None, symm or None)."""
        natoms = np.array([s.posn.shape[0] for s in structures], dtype=np.int32)
        posn = np.ascontiguousarray(np.concatenate([np.asarray(s.posn, dtype=np.float64) for s in structures]) if len(structures) else np.zeros((0, 3)))
        species = np.ascontiguousarray(np.concatenate([np.asarray(s.species, dtype=np.int32) for s in structures]) if len(structures) else np.zeros(0, np.int32))
        cell = np.ascontiguousarray(np.concatenate([_cell_colmajor(s.cell) for s in structures]) if len(structures) else np.zeros(0))
        n = int(natoms.sum())
        energy = np.zeros(len(structures)) if flags & ENERGY else None
        force = np.zeros((n, 3)) if flags & FORCE else None
        symm = np.zeros((n, max(self.ninput)), dtype=np.float32) if flags & SYMM else None
        self._check(self.lib.nnpgpu_compute(self._ctx, len(structures), _p(natoms), _p(posn), _p(species), _p(cell), flags, _p(energy),
                                            _p(force), _p(symm)))
        forces = None
        if force is not None:
            offs = np.concatenate([[0], np.cumsum(natoms)])
            forces = [force[offs[k]:offs[k + 1]] for k in range(len(structures))]
        return energy, forces, symm

    def compute_flat(self, natoms, posn, species, cells_colmajor, flags, energy=None, force=None, symm=None):
        """nnpgpu_compute on pre-packed host arrays (outputs written in place)."""
        self._check(self.lib.nnpgpu_compute(self._ctx, len(natoms), _p(natoms), _p(posn), _p(species), _p(cells_colmajor), flags,
                                            _p(energy), _p(force), _p(symm)))

    def compute_device(self, natoms, d_posn, d_species, cells_colmajor, flags, d_energy=0, d_force=0, d_symm=0, stream=0):
        """Device-resident variant: d_* are raw device pointers (ints), natoms and cells host arrays."""
        natoms = np.ascontiguousarray(natoms, dtype=np.int32)
        cells = np.ascontiguousarray(cells_colmajor, dtype=np.float64)
        self._check(self.lib.nnpgpu_compute_device(self._ctx, len(natoms), _p(natoms), ctypes.c_void_p(d_posn),
                                                   ctypes.c_void_p(d_species), _p(cells), flags, ctypes.c_void_p(d_energy or None),
                                                   ctypes.c_void_p(d_force or None), ctypes.c_void_p(d_symm or None),
                                                   ctypes.c_void_p(stream or None)))

    def symm_noalloc(self, natoms, d_posn, d_species, cell, d_symm, symm_stride, stream=0):
        """nnpgpu_symm_noalloc: symmetry functions of one structure with no device allocation
        (device pointers in and out; cell is a 3x3 host array, columns = lattice vectors)."""
        cellc = _cell_colmajor(cell)
        self._check(self.lib.nnpgpu_symm_noalloc(self._ctx, natoms, ctypes.c_void_p(d_posn or None), ctypes.c_void_p(d_species or None),
                                                 _p(cellc), ctypes.c_void_p(d_symm or None), symm_stride, ctypes.c_void_p(stream or None)))

    # ---- launch-shape autotuner
    def autotune(self, natoms, posn, species, cells_colmajor, flags=FORCE):
        """nnpgpu_autotune on pre-packed host arrays; returns (shapes dict, report string)."""
        buf = ctypes.create_string_buffer(4096)
        natoms = np.ascontiguousarray(natoms, dtype=np.int32)
        self._check(self.lib.nnpgpu_autotune(self._ctx, len(natoms), _p(natoms), _p(np.ascontiguousarray(posn, dtype=np.float64)),
                                             _p(np.ascontiguousarray(species, dtype=np.int32)),
                                             _p(np.ascontiguousarray(cells_colmajor, dtype=np.float64)), flags, buf, len(buf)))
        return self.get_tune(), buf.value.decode()

    def get_tune(self):
        v = [ctypes.c_int() for _ in range(4)]
        self._check(self.lib.nnpgpu_get_tune(self._ctx, *[ctypes.byref(x) for x in v]))
        return dict(zip(("warps_nbr", "warps_symm", "warps_force", "nn_tile"), (x.value for x in v)))

    def set_tune(self, warps_nbr=4, warps_symm=4, warps_force=4, nn_tile=32):
        self._check(self.lib.nnpgpu_set_tune(self._ctx, warps_nbr, warps_symm, warps_force, nn_tile))

    def set_wait_limit(self, polls=1 << 22):
        """nnpgpu_set_wait_limit: polls of each mbarrier wait of the tensor-core networks."""
        self._check(self.lib.nnpgpu_set_wait_limit(self._ctx, polls))

    # ---- training: batch error and parameter gradient of the energy loss
    LOSS = {"MSE": 0, "MAE": 1, "HUBER": 2, "ASINH": 3}

    def nparams(self, t):
        return self.lib.nnpgpu_nparams(self._ctx, t)

    def train_grad(self, structures, energy_ref, loss="MSE", delta=1.0):
        """(sum of losses, sum of dE^2, gradient) of one batch (nnpgpu_train_grad)."""
        natoms = np.array([s.posn.shape[0] for s in structures], dtype=np.int32)
        posn = np.ascontiguousarray(np.concatenate([np.asarray(s.posn, dtype=np.float64) for s in structures]))
        species = np.ascontiguousarray(np.concatenate([np.asarray(s.species, dtype=np.int32) for s in structures]))
        cell = np.ascontiguousarray(np.concatenate([_cell_colmajor(s.cell) for s in structures]))
        eref = np.ascontiguousarray(energy_ref, dtype=np.float64)
        err = np.zeros(2)
        grad = np.zeros(sum(self.nparams(t) for t in range(self.ntypes)))
        self._check(self.lib.nnpgpu_train_grad(self._ctx, len(structures), _p(natoms), _p(posn), _p(species), _p(cell), _p(eref),
                                               self.LOSS[loss], float(delta), _p(err), _p(grad)))
        return err[0], err[1], grad

    def train_force_grad(self, structures, energy_ref, force_ref, beta, loss="MSE", delta=1.0):
        """(loss, sum of dE^2, sum of |dF/N|^2, gradient) of one batch with forces
        (nnpgpu_train_force_grad); force_ref: one (N,3) array per structure."""
        natoms = np.array([s.posn.shape[0] for s in structures], dtype=np.int32)
        posn = np.ascontiguousarray(np.concatenate([np.asarray(s.posn, dtype=np.float64) for s in structures]))
        species = np.ascontiguousarray(np.concatenate([np.asarray(s.species, dtype=np.int32) for s in structures]))
        cell = np.ascontiguousarray(np.concatenate([_cell_colmajor(s.cell) for s in structures]))
        eref = np.ascontiguousarray(energy_ref, dtype=np.float64)
        fref = np.ascontiguousarray(np.concatenate([np.asarray(f, dtype=np.float64) for f in force_ref]))
        err = np.zeros(3)
        grad = np.zeros(sum(self.nparams(t) for t in range(self.ntypes)))
        self._check(self.lib.nnpgpu_train_force_grad(self._ctx, len(structures), _p(natoms), _p(posn), _p(species), _p(cell), _p(eref),
                                                     _p(fref), float(beta), self.LOSS[loss], float(delta), _p(err), _p(grad)))
        return err[0], err[1], err[2], grad

    def params(self, t):
        """Network parameters of species t (nnpgpu_get_params; biases, then weights input-outer)."""
        p = np.zeros(self.nparams(t))
        self._check(self.lib.nnpgpu_get_params(self._ctx, t, _p(p)))
        return p

    def set_params(self, t, p):
        """Replace the network parameters of species t (nnpgpu_set_params)."""
        p = np.ascontiguousarray(p, dtype=np.float64)
        if p.size != self.nparams(t):
            raise ValueError("species %d has %d parameters" % (t, self.nparams(t)))
        self._check(self.lib.nnpgpu_set_params(self._ctx, t, _p(p)))

    def write_potential(self, path):
        """The potential with its current parameters in the reference's text format."""
        self._check(self.lib.nnpgpu_write_potential(self._ctx, path.encode()))

    def energy_symm(self, natoms, species, symm, flags=0):
        """Energies of structures from stored descriptors (nnpgpu_energy_symm): natoms per
        structure, species and symm rows (FP64, at least the largest input size wide) of all
        their atoms concatenated."""
        natoms = np.ascontiguousarray(natoms, dtype=np.int32)
        species = np.ascontiguousarray(species, dtype=np.int32)
        symm = np.ascontiguousarray(symm, dtype=np.float64)
        energy = np.zeros(len(natoms))
        self._check(self.lib.nnpgpu_energy_symm(self._ctx, len(natoms), _p(natoms), _p(species), _p(symm), symm.shape[1], int(flags),
                                                _p(energy)))
        return energy

    # ---- molecular dynamics on resident device state
    def md(self, struc, mass, dt, skin=1.0, vel=None, flags=0):
        """An MD run of one structure (nnpgpu_md_*); mass per atom.  Returns an MD object."""
        return MD(self, struc, mass, dt, skin, vel, flags)

    # ---- serving (continuous batching)
    def serve_start(self, max_batch_atoms=0, max_inflight=2, hbm_budget_bytes=0, skin=1.0, flags=0):
        o = ServeOpts(max_batch_atoms, max_inflight, hbm_budget_bytes, skin, flags)
        self._check(self.lib.nnpgpu_serve_start(self._ctx, ctypes.byref(o)))

    def submit(self, struc, key=-1):
        posn = np.ascontiguousarray(struc.posn, dtype=np.float64)
        species = np.ascontiguousarray(struc.species, dtype=np.int32)
        rid = ctypes.c_longlong()
        self._check(self.lib.nnpgpu_submit(self._ctx, posn.shape[0], _p(posn), _p(species), _p(_cell_colmajor(struc.cell)), key,
                                           ctypes.byref(rid)))
        return rid.value

    def poll(self, rid, natoms):
        """(energy, forces, latency_s) when done, None while pending."""
        e = np.zeros(1)
        F = np.zeros((natoms, 3))
        lat = ctypes.c_double()
        rc = self.lib.nnpgpu_poll(self._ctx, rid, _p(e), _p(F), ctypes.byref(lat))
        if rc == ERR_BUSY:
            return None
        self._check(rc)
        return float(e[0]), F, lat.value

    def serve_stop(self):
        self._check(self.lib.nnpgpu_serve_stop(self._ctx))

    def profile_enable(self, on=True):
        self._check(self.lib.nnpgpu_profile_enable(self._ctx, 1 if on else 0))

    def profile_read(self):
        """{stage name: (total ms, count)} of the batched launch sequence since profile_enable."""
        out = {}
        for k in range(6):
            ms, n = ctypes.c_double(), ctypes.c_longlong()
            self._check(self.lib.nnpgpu_profile_read(self._ctx, k, ctypes.byref(ms), ctypes.byref(n)))
            out[self.lib.nnpgpu_profile_stage_name(k).decode()] = (ms.value, n.value)
        return out

    def neighbors(self, posn, cell, cap=256, rc=None):
        """Neighbour list of one structure built on the GPU (reference list order), at the
        potential's cutoff or at ``rc``."""
        posn = np.ascontiguousarray(posn, dtype=np.float64)
        n = posn.shape[0]
        count = np.zeros(n, dtype=np.int32)
        index = np.zeros((n, cap), dtype=np.int32)
        r = np.zeros((n, cap, 4), dtype=np.float32)
        mn = np.zeros((n, cap), dtype=np.uint8)
        sh = np.zeros((n, cap, 3), dtype=np.int32)
        if rc is None:
            self._check(self.lib.nnpgpu_neighbors(self._ctx, n, _p(posn), _p(_cell_colmajor(cell)), cap, _p(count), _p(index), _p(r),
                                                  _p(mn), _p(sh)))
        else:
            self._check(self.lib.nnpgpu_neighbors_rc(self._ctx, float(rc), n, _p(posn), _p(_cell_colmajor(cell)), cap, _p(count),
                                                     _p(index), _p(r), _p(mn), _p(sh)))
        return [dict(index=index[i, :count[i]].copy(), r=r[i, :count[i], :3].astype(np.float64), dr=r[i, :count[i], 3].astype(np.float64),
                     min=mn[i, :count[i]].astype(bool), shift=sh[i, :count[i]].copy()) for i in range(n)]


class MD:
    """Velocity-Verlet MD with the engine's forces, state resident on the GPU (nnpgpu_md_*)."""

    def __init__(self, eng, struc, mass, dt, skin=1.0, vel=None, flags=0):
        self.eng = eng
        self.n = struc.posn.shape[0]
        posn = np.ascontiguousarray(struc.posn, dtype=np.float64)
        species = np.ascontiguousarray(struc.species, dtype=np.int32)
        mass = np.ascontiguousarray(np.broadcast_to(np.asarray(mass, dtype=np.float64), (self.n,)))
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
        h = ctypes.c_void_p()
        eng._check(eng.lib.nnpgpu_md_create(eng._ctx, self.n, _p(posn), _p(v), _p(species), _p(mass), _p(_cell_colmajor(struc.cell)),
                                            float(dt), float(skin), flags, ctypes.byref(h)))
        self._h = h

    def forces(self):
        pe = np.zeros(1)
        self.eng._check(self.eng.lib.nnpgpu_md_forces(self._h, _p(pe)))
        return float(pe[0])

    def run(self, nsteps):
        pe, ke = np.zeros(nsteps), np.zeros(nsteps)
        self.eng._check(self.eng.lib.nnpgpu_md_run(self._h, nsteps, _p(pe), _p(ke)))
        return pe, ke

    def state(self):
        x, v, F = np.zeros((self.n, 3)), np.zeros((self.n, 3)), np.zeros((self.n, 3))
        nb = ctypes.c_int()
        self.eng._check(self.eng.lib.nnpgpu_md_state(self._h, _p(x), _p(v), _p(F), ctypes.byref(nb)))
        return x, v, F, nb.value

    def close(self):
        if self._h:
            self.eng.lib.nnpgpu_md_destroy(self._h)
            self._h = None
