"""ctypes binding of the FP64 CPU oracle (oracle/_build/libnnp_oracle.so).

TEST INFRASTRUCTURE ONLY: used by the tests, the smoke check and the CPU-baseline leg of
bench.py, as the checker.  Parity status: unpinned against the reference binary, which cannot
be built here; pinned by the reference tests' properties (see nnp_oracle.h).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libnnp_oracle.so")
_lib = None

ENERGY, FORCE, COMPUTE = 1, 2, 4


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, ip, dp, cp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_char_p
        L.oracle_nnp_read.restype = vp
        L.oracle_nnp_read.argtypes = [cp, cp, ip]
        L.oracle_nnp_free.argtypes = [vp]
        L.oracle_nnp_ntypes.argtypes = [vp]
        L.oracle_nnp_ninput.argtypes = [vp, ip]
        L.oracle_nnp_rc.argtypes = [vp]
        L.oracle_nnp_rc.restype = dp
        L.oracle_nnp_type_index.argtypes = [vp, cp]
        L.oracle_nnp_write.argtypes = [vp, cp]
        L.oracle_neighbors.argtypes = [dp, ip, vp, vp, ip, vp, vp, vp, vp, vp, vp]
        L.oracle_compute.argtypes = [vp, ip, vp, vp, vp, ip, vp, vp, vp, ip]
        L.oracle_network.argtypes = [vp, ip, vp, vp]
        L.oracle_compute_centres.argtypes = [vp, ip, vp, vp, vp, ip, vp, vp]
        L.oracle_network.restype = dp
        L.oracle_nnp_nparams.argtypes = [vp, ip]
        L.oracle_train_grad.argtypes = [vp, ip, vp, vp, ip, vp, vp, ip, dp, vp, vp]
        L.oracle_nnp_get_params.argtypes = [vp, ip, vp]
        L.oracle_nnp_get_params.restype = None
        L.oracle_nnp_set_params.argtypes = [vp, ip, vp]
        L.oracle_nnp_set_params.restype = None
        L.oracle_train_force_grad.argtypes = [vp, ip, vp, vp, vp, vp, vp, vp, dp, ip, dp, vp, vp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class OracleNNP:
    """A potential loaded by the oracle (NNP::read, src/nnp/nnp.cpp:244-308)."""

    def __init__(self, path):
        err = ctypes.create_string_buffer(512)
        self._h = lib().oracle_nnp_read(path.encode(), err, 512)
        if not self._h:
            raise RuntimeError("oracle could not read %s: %s" % (path, err.value.decode()))
        self.ntypes = lib().oracle_nnp_ntypes(self._h)
        self.rc = lib().oracle_nnp_rc(self._h)
        self.ninput = [lib().oracle_nnp_ninput(self._h, t) for t in range(self.ntypes)]

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_nnp_free(self._h)
            self._h = None

    def type_index(self, name):
        return lib().oracle_nnp_type_index(self._h, name.encode())

    def write(self, path):
        if lib().oracle_nnp_write(self._h, path.encode()) != 0:
            raise RuntimeError("oracle could not write " + path)

    def compute(self, posn, species, cell, force=True, compute_semantics=False, symm=False):
        """Returns (energy, forces (N,3) or None, symm (N, max ninput) or None)."""
        posn = np.ascontiguousarray(posn, dtype=np.float64)
        species = np.ascontiguousarray(species, dtype=np.int32)
        cellc = None if cell is None else np.ascontiguousarray(np.asarray(cell, dtype=np.float64).T).ravel()
        n = posn.shape[0]
        e = np.zeros(1)
        F = np.zeros((n, 3)) if force or compute_semantics else None
        stride = max(self.ninput)
        G = np.zeros((n, stride)) if symm else None
        flags = COMPUTE if compute_semantics else (ENERGY | (FORCE if force else 0))
        rc = lib().oracle_compute(self._h, n, _ptr(posn), _ptr(species), _ptr(cellc), flags, _ptr(e), _ptr(F),
                                  _ptr(G), stride)
        if rc != 0:
            raise RuntimeError("oracle_compute failed (%d)" % rc)
        return float(e[0]), F, G

    def compute_centres(self, posn, species, cell, centres):
        """E+F work of the listed centre atoms only (timing samples of large cells); returns the
        centres' atomic energies summed (vacuum energies included)."""
        posn = np.ascontiguousarray(posn, dtype=np.float64)
        species = np.ascontiguousarray(species, dtype=np.int32)
        centres = np.ascontiguousarray(centres, dtype=np.int32)
        cellc = None if cell is None else np.ascontiguousarray(np.asarray(cell, dtype=np.float64).T).ravel()
        e = np.zeros(1)
        rc = lib().oracle_compute_centres(self._h, posn.shape[0], _ptr(posn), _ptr(species), _ptr(cellc), len(centres), _ptr(centres), _ptr(e))
        if rc != 0:
            raise RuntimeError("oracle_compute_centres failed (%d)" % rc)
        return float(e[0])

    def train_grad(self, structures, energy_ref, loss=0, delta=1.0):
        """The energy trainer's batch error and gradient (NNPTE::error, src/nnp/nnpte.cpp:870-921) on
        the oracle's own FP64 symmetry functions: (sum of losses, sum of dE^2, gradient)."""
        rows, types, natoms = [], [], []
        stride = max(self.ninput)
        for s in structures:
            _, _, G = self.compute(s.posn, s.species, s.cell, force=False, symm=True)
            rows.append(G)
            types.append(np.asarray(s.species, dtype=np.int32))
            natoms.append(s.posn.shape[0])
        symm = np.ascontiguousarray(np.concatenate(rows))
        types = np.ascontiguousarray(np.concatenate(types))
        natoms = np.asarray(natoms, dtype=np.int32)
        eref = np.ascontiguousarray(energy_ref, dtype=np.float64)
        err = np.zeros(2)
        grad = np.zeros(sum(lib().oracle_nnp_nparams(self._h, t) for t in range(self.ntypes)))
        rc = lib().oracle_train_grad(self._h, len(natoms), _ptr(natoms), _ptr(symm), stride, _ptr(types), _ptr(eref), int(loss),
                                     float(delta), _ptr(err), _ptr(grad))
        if rc != 0:
            raise RuntimeError("oracle_train_grad failed (%d)" % rc)
        return err[0], err[1], grad

    def params(self, t):
        """Network parameters of type t in the reference's order (biases, then weights input-outer)."""
        p = np.zeros(lib().oracle_nnp_nparams(self._h, t))
        lib().oracle_nnp_get_params(self._h, t, _ptr(p))
        return p

    def set_params(self, t, p):
        p = np.ascontiguousarray(p, dtype=np.float64)
        assert p.size == lib().oracle_nnp_nparams(self._h, t)
        lib().oracle_nnp_set_params(self._h, t, _ptr(p))

    def train_force_grad(self, structures, energy_ref, force_ref, beta, loss=0, delta=1.0):
        """The force trainer's batch error and exact gradient (loss of NNPTEF::error,
        src/nnp/nnptef.cpp:1043-1135): (loss, sum of dE^2, sum of |dF/N|^2, gradient)."""
        natoms = np.asarray([s.posn.shape[0] for s in structures], dtype=np.int32)
        posn = np.ascontiguousarray(np.concatenate([np.asarray(s.posn, np.float64) for s in structures]))
        types = np.ascontiguousarray(np.concatenate([np.asarray(s.species, np.int32) for s in structures]))
        cells = np.ascontiguousarray(np.concatenate([np.asarray(s.cell, np.float64).T.ravel() for s in structures]))
        eref = np.ascontiguousarray(energy_ref, dtype=np.float64)
        fref = np.ascontiguousarray(np.concatenate([np.asarray(f, np.float64) for f in force_ref]))
        err = np.zeros(3)
        grad = np.zeros(sum(lib().oracle_nnp_nparams(self._h, t) for t in range(self.ntypes)))
        rc = lib().oracle_train_force_grad(self._h, len(natoms), _ptr(natoms), _ptr(posn), _ptr(types), _ptr(cells), _ptr(eref),
                                           _ptr(fref), float(beta), int(loss), float(delta), _ptr(err), _ptr(grad))
        if rc != 0:
            raise RuntimeError("oracle_train_force_grad failed (%d)" % rc)
        return err[0], err[1], err[2], grad

    def network(self, t, g):
        g = np.ascontiguousarray(g, dtype=np.float64)
        d = np.zeros_like(g)
        out = lib().oracle_network(self._h, t, _ptr(g), _ptr(d))
        return out, d


def neighbors(rc, posn, cell, cap=512):
    """Neighbour list of one structure in the reference's order (NeighborList::build,
    src/struc/neighbor.cpp:59-171).  Returns a list (per atom) of dicts of arrays."""
    posn = np.ascontiguousarray(posn, dtype=np.float64)
    cellc = None if cell is None else np.ascontiguousarray(np.asarray(cell, dtype=np.float64).T).ravel()
    n = posn.shape[0]
    while True:
        count = np.zeros(n, dtype=np.int32)
        index = np.zeros((n, cap), dtype=np.int32)
        r = np.zeros((n, cap, 3))
        dr = np.zeros((n, cap))
        mn = np.zeros((n, cap), dtype=np.uint8)
        sh = np.zeros((n, cap, 3), dtype=np.int32)
        rcode = lib().oracle_neighbors(rc, n, _ptr(posn), _ptr(cellc), cap, _ptr(count), _ptr(index), _ptr(r),
                                       _ptr(dr), _ptr(mn), _ptr(sh))
        if rcode == -1:
            cap = int(count.max()) + 8
            continue
        if rcode != 0:
            raise RuntimeError("oracle_neighbors failed")
        return [dict(index=index[i, :count[i]].copy(), r=r[i, :count[i]].copy(), dr=dr[i, :count[i]].copy(),
                     min=mn[i, :count[i]].astype(bool), shift=sh[i, :count[i]].copy()) for i in range(n)]
