/*
 * nnp_oracle.h - C interface of the FP64 CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C++ FP64 restatement of AtomNN's
 * Behler-Parrinello energy/force path (neighbour list, G2/G4 symmetry functions,
 * atomic networks, chain-rule forces).  Only the tests, the smoke check and the
 * CPU-baseline leg of bench.py load it, as the checker.  The product path never
 * links it.
 *
 * Parity status: unpinned against the reference binary.  The reference cannot be
 * compiled here (Eigen 3.4 and MPI are absent, and src/nnp/nnp_compute.cpp is
 * missing from the snapshot) and its tests hold no golden vectors.  The oracle is
 * pinned instead by the properties the reference's own tests check: supercell
 * invariance of G and E/atom (src/nnp/test_nnp_symm.cpp:292-501), neighbour
 * displacements contained in the supercell list (src/struc/test_neigh_unit.cpp:14-109),
 * and finite-difference derivatives (src/nnp/test_basis_radial.cpp:15-67,
 * src/nnp/test_basis_angular.cpp:17-130, src/nnp/test_cutoff.cpp:20-58).
 */
#ifndef NNP_ORACLE_H
#define NNP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* flags for oracle_compute */
#define ORACLE_ENERGY 1   /* NNP::energy  (src/nnp/nnp.cpp:390-402), includes vacuum energy */
#define ORACLE_FORCE  2   /* NNP::force   (src/nnp/nnp.cpp:416-482) */
#define ORACLE_COMPUTE 4  /* NNP::compute (src/nnp/nnp.cpp:496-566), energy WITHOUT vacuum energy */

/* Reads a potential in the reference text format (NNP::read, src/nnp/nnp.cpp:244-308).
 * Returns an opaque handle or NULL; on failure err receives a message. */
void* oracle_nnp_read(const char* path, char* err, int errlen);
void oracle_nnp_free(void* nnp);
int oracle_nnp_ntypes(const void* nnp);
int oracle_nnp_ninput(const void* nnp, int type);
double oracle_nnp_rc(const void* nnp);
int oracle_nnp_type_index(const void* nnp, const char* name);
/* Writes the potential back in the reference text format (NNP::write, src/nnp/nnp.cpp:198-237). */
int oracle_nnp_write(const void* nnp, const char* path);

/* Neighbour list of one structure (NeighborList::build, src/struc/neighbor.cpp:59-171).
 * cell: 9 doubles, column-major (columns are the lattice vectors); NULL or all-zero for
 * a non-periodic structure.  posn: natoms*3.  For every atom at most cap entries are
 * written, in the reference's list order.  Per entry: index (neighbour atom), r (3 doubles,
 * vector from the neighbour to the centre), dr, min flag, and shift (3 ints: the integer
 * lattice translation T with r = posn_i - posn_j - R*T).
 * Returns 0, or -1 if some atom has more than cap neighbours (count still holds the true sizes). */
int oracle_neighbors(double rc, int natoms, const double* posn, const double* cell, int cap,
                     int* count, int* index, double* r, double* dr, unsigned char* min, int* shift);

/* Full evaluation of one structure, as the compute tool does (src/nnp/nnpce.cpp:273-281):
 * neighbour list, NNP::symm, then NNP::energy and/or NNP::force, or NNP::compute.
 * type: per-atom index into the potential's types.  energy: 1 double.  force: natoms*3 or NULL.
 * symm: natoms*symm_stride doubles or NULL.  Returns 0 or a negative error code. */
int oracle_compute(void* nnp, int natoms, const double* posn, const int* type, const double* cell,
                   int flags, double* energy, double* force, double* symm, int symm_stride);

/* Energy and dE/dG of one atomic network (ANN::fpbp + DODZ::grad, src/ml/nn.cpp:1215-1233,1620-1628).
 * Returns the network output (without vacuum energy). */
double oracle_network(void* nnp, int type, const double* symm, double* dedg);
// E+F work of a subset of centre atoms (lists scanning every atom, descriptors, networks, chain
// rule), for timing samples of large structures; energy = the centres' network outputs + vacuum
int oracle_compute_centres(void* nnp, int natoms, const double* posn, const int* type, const double* cell, int ncentre,
                           const int* centres, double* energy);
/* network parameters of a type (ANN::size) and the energy trainer's batch error and gradient */
int oracle_nnp_nparams(const void* nnp, int type);
int oracle_train_grad(void* nnp, int nstruc, const int* natoms, const double* symm, int stride, const int* type,
                      const double* eref, int loss, double delta, double* error, double* grad);
/* network parameters in the reference's order, and the force trainer's batch error and exact
 * gradient (loss of src/nnp/nnptef.cpp:1043-1135; see nnp_oracle.cpp) */
void oracle_nnp_get_params(const void* nnp, int type, double* p);
void oracle_nnp_set_params(void* nnp, int type, const double* p);
int oracle_train_force_grad(void* nnp, int nstruc, const int* natoms, const double* posn, const int* type, const double* cells,
                            const double* eref, const double* fref, double beta, int loss, double delta, double* error, double* grad);

#ifdef __cplusplus
}
#endif
#endif
