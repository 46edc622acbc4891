/*
 * nnpgpu.h - C ABI of the GB300 energy/force engine for Behler-Parrinello potentials.
 *
 * Drop-in boundary for the NNP energy/force calls of AtomNN (markdellostritto/AtomNN).
 * The reference exposes static C++ functions on class NNP (src/nnp/nnp.hpp:108-120) plus
 * NeighborList::build (src/struc/neighbor.hpp:85); those are not callable through an FFI,
 * so each entry point below names the reference call(s) it replaces.  Plain pointers and
 * sizes only; every function returns a status code (0 = ok) instead of throwing, and the
 * message of the last failure is available from nnpgpu_last_error().
 *
 * Units are the potential's (metal: Angstrom, eV).  Cells are 9 doubles, column-major, the
 * columns being the lattice vectors (Cell::R_, src/struc/cell.hpp); an all-zero cell means a
 * non-periodic structure.  Positions are Cartesian, natoms*3 doubles.  Species are indices
 * into the potential's type list (what NNP::index(name) returns, src/nnp/nnp.hpp:83).
 *
 * Threading: one context per host thread; a context owns its CUDA stream and device memory.
 */
#ifndef NNPGPU_H
#define NNPGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define NNPGPU_OK 0
#define NNPGPU_ERR_INVALID (-1)     /* invalid argument or input (NaN position, bad species, singular cell, a force
                                       contribution that is not finite or above 1e9 eV/A) */
#define NNPGPU_ERR_IO (-2)          /* potential file could not be read (NNP::read throws, src/nnp/nnp.cpp:190) */
#define NNPGPU_ERR_CUDA (-3)        /* CUDA runtime error, or no usable GPU */
#define NNPGPU_ERR_OOM (-4)         /* device allocation failed or the HBM budget would be exceeded */
#define NNPGPU_ERR_CAPACITY (-5)    /* neighbour capacity exceeded after the automatic retry */
#define NNPGPU_ERR_TIMEOUT (-6)     /* a bounded wait on the device ran out */
#define NNPGPU_ERR_UNSUPPORTED (-7) /* potential uses a form the GPU kernels do not implement */
#define NNPGPU_ERR_BUSY (-8)        /* serving: request not finished yet, or queue full */

/* flags for nnpgpu_compute */
#define NNPGPU_ENERGY 0x1     /* energy per structure (NNP::energy, src/nnp/nnp.cpp:390-402) */
#define NNPGPU_FORCE 0x2      /* forces (NNP::force, src/nnp/nnp.cpp:416-482) */
#define NNPGPU_SYMM 0x4       /* symmetry functions (NNP::symm, src/nnp/nnp.cpp:334-381), FP32 */
#define NNPGPU_BF16 0x8       /* atomic networks as BF16 tensor-core GEMMs (FP32 accumulate) */
#define NNPGPU_NO_VACUUM 0x10 /* energy without the species vacuum energy (NNP::compute, src/nnp/nnp.cpp:496-566) */
#define NNPGPU_BATCHED 0x20   /* all structures in one launch sequence; otherwise one structure at a time */

typedef struct nnpgpu_ctx nnpgpu_ctx;

typedef struct nnpgpu_opts {
  int device;              /* CUDA device ordinal */
  int max_neighbors;       /* initial neighbour capacity per atom (0 = estimate from density); grows on overflow */
  size_t hbm_budget_bytes; /* cap on the context's device memory (0 = no cap) */
  int verbose;
} nnpgpu_opts;

/* Reads a potential file in AtomNN's text format and prepares the device.
 * Replaces NNP::read(const char*, NNP&) (src/nnp/nnp.cpp:182-191,244-308). */
int nnpgpu_create(const char* potfile, const nnpgpu_opts* opts, nnpgpu_ctx** out);
void nnpgpu_destroy(nnpgpu_ctx* ctx);
const char* nnpgpu_last_error(const nnpgpu_ctx* ctx);

/* Potential queries: NNP::ntypes (nnp.hpp:82), NNP::index(name) (nnp.hpp:83),
 * NNP::rc (nnp.hpp:90), NNH::nInput (nnh.hpp:91). */
int nnpgpu_ntypes(const nnpgpu_ctx* ctx);
int nnpgpu_type_index(const nnpgpu_ctx* ctx, const char* name);
double nnpgpu_cutoff(const nnpgpu_ctx* ctx);
int nnpgpu_ninput(const nnpgpu_ctx* ctx, int type);

/* Energy, forces and/or symmetry functions of nstruc structures (host buffers).
 * Replaces the compute tool's per-structure sequence NeighborList::build + NNP::symm +
 * NNP::energy + NNP::force (src/nnp/nnpce.cpp:273-281), or NNP::compute with NNPGPU_NO_VACUUM.
 *   natoms[nstruc], posn[sum(natoms)*3], species[sum(natoms)], cell[nstruc*9]
 *   energy[nstruc] (FP64) if NNPGPU_ENERGY, force[sum(natoms)*3] (FP64) if NNPGPU_FORCE,
 *   symm[sum(natoms)*max_ninput] (FP32, row stride = max over types of nnpgpu_ninput) if NNPGPU_SYMM. */
int nnpgpu_compute(nnpgpu_ctx* ctx, int nstruc, const int* natoms, const double* posn, const int* species,
                   const double* cell, int flags, double* energy, double* force, float* symm);

/* Same computation on device-resident data: posn, species, energy, force, symm are device
 * pointers; natoms and cell stay on the host.  stream is a cudaStream_t (NULL = the context's
 * stream).  Returns after the stream has finished the work: the status words are read back so
 * that a neighbour-capacity overflow is retried inside the call. */
int nnpgpu_compute_device(nnpgpu_ctx* ctx, int nstruc, const int* natoms, const double* d_posn,
                          const int* d_species, const double* cell, int flags, double* d_energy,
                          double* d_force, float* d_symm, void* stream);

/* Neighbour list of one structure, built on the GPU.  Replaces NeighborList::build
 * (src/struc/neighbor.cpp:59-171).  Per atom at most cap entries in the reference's order:
 * index (neighbour atom), r[4] = (x, y, z, |r|) FP32 with r pointing from the neighbour to the
 * centre, min flag, shift[3] = integer lattice translation T (r = posn_i - posn_j - R*T).
 * count[natoms] receives the full sizes; returns NNPGPU_ERR_CAPACITY if some count > cap. */
int nnpgpu_neighbors(nnpgpu_ctx* ctx, int natoms, const double* posn, const double* cell, int cap,
                     int* count, int* index, float* r, unsigned char* min, int* shift);

/* The same at an explicit cutoff rc > 0 (NeighborList::build(const Structure&, double rc),
 * src/struc/neighbor.hpp:85, whose cutoff is the caller's and need not be the potential's), with
 * up to 1024 entries per atom.  The context only provides the device and its stream. */
int nnpgpu_neighbors_rc(nnpgpu_ctx* ctx, double rc, int natoms, const double* posn, const double* cell,
                        int cap, int* count, int* index, float* r, unsigned char* min, int* shift);

/* ---- symmetry functions without device allocation.  This entry point has no counterpart in the
 * reference.  It is for callers that cannot let a library allocate device memory while they run:
 * codes that divide the GPU's memory among their own pools before the first step, and services
 * that reserve all device memory at start-up, where an allocation in the middle of a step could
 * fail or synchronise the device at a point the caller does not control.  It computes the same
 * symmetry functions as nnpgpu_compute with NNPGPU_SYMM, for one structure of at most 1024 atoms
 * with at most 192 neighbours per atom and 512 lattice images, and keeps every intermediate in a
 * 4.6 MB scratch array compiled into the library (each GPU that loads the library holds it until
 * the process exits).  It calls no cudaMalloc, cudaFree or allocating library routine.
 * d_posn (natoms*3 FP64), d_species and d_symm (natoms rows of symm_stride FP32, symm_stride >= the
 * largest nnpgpu_ninput) are device pointers; cell is a host array as in nnpgpu_compute.  Returns
 * after the work on stream (NULL = the context's stream) has finished.  Larger requests are
 * rejected with NNPGPU_ERR_INVALID or NNPGPU_ERR_CAPACITY and a message.
 * Set-up: the first call on a context (natoms = 0 is enough) looks up the scratch array's device
 * address and loads the kernels this entry point launches (CUDA loads them lazily, and loading
 * places code in device memory); make that call before reserving the device's memory and before
 * any stream capture.  All calls share the scratch array, so calls whose work overlaps on the GPU
 * race on it: serialise them.  The caller's current device is left as it was. */
int nnpgpu_symm_noalloc(nnpgpu_ctx* ctx, int natoms, const double* d_posn, const int* d_species, const double* cell,
                        float* d_symm, int symm_stride, void* stream);

/* ---- stage tracing (diagnostics; the reference times phases with util/Clock, e.g.
 * src/nnp/nnpte.cpp:1971-1990).  When enabled, CUDA events bracket each stage of the batched
 * launch sequence and their durations accumulate per stage.  Enabling resets the counters. */
#define NNPGPU_NSTAGES 6 /* 0 neighbours, 1 clearing of the force sums, 2 descriptors, 3 networks, 4 chain rule, 5 forces+energy */
int nnpgpu_profile_enable(nnpgpu_ctx* ctx, int on);
int nnpgpu_profile_read(const nnpgpu_ctx* ctx, int stage, double* total_ms, long long* count);
const char* nnpgpu_profile_stage_name(int stage);

/* ---- energies from stored descriptors: NNP::energy on struc.symm() (src/nnp/nnp.cpp:390-402, the
 * network pass ANN::fp of src/ml/nn.cpp:1191-1209), as the trainers use it on descriptors read
 * back from a binary structure file (Structure::read_binary, src/struc/structure.cpp:155-190).
 * No neighbour list and no descriptor pass: symm[sum(natoms)][symm_stride] (FP64, row-major;
 * atom i's first nnpgpu_ninput(ctx, species[i]) values are used, symm_stride >= every input
 * size); flags: NNPGPU_BF16, NNPGPU_NO_VACUUM; energy[nstruc] (FP64).  The networks run in FP32
 * (or BF16) on the descriptors rounded to FP32. */
int nnpgpu_energy_symm(nnpgpu_ctx* ctx, int nstruc, const int* natoms, const int* species, const double* symm,
                       int symm_stride, int flags, double* energy);

/* ---- training: the energy trainer's batch error and parameter gradient.  Replaces the error and
 * gradient part of NNPTE::error (src/nnp/nnpte.cpp:870-921) with Cost::grad (src/ml/nn.cpp:1554-1589):
 * per structure E = sum of the atomic network outputs (no vacuum energies), dE = (E - E_ref)/N and
 * loss 0 MSE dE^2/2, 1 MAE |dE|, 2 HUBER delta^2 (sqrt(1 + (dE/delta)^2) - 1),
 * 3 ASINH delta^2 (1 - sqrt(1 + x^2) + x asinh x), x = dE/delta.
 *   energy_ref[nstruc]; error[0] = sum of the losses, error[1] = sum of dE^2;
 *   grad = the gradient of sum of losses, per species nnpgpu_nparams(ctx, t) values concatenated in
 *   species order, each in the reference's parameter order (every layer's biases, then every
 *   layer's weights with the input index outer and the node index inner).
 * Descriptors are computed from the positions on each call (FP32, FP32 networks). */
int nnpgpu_nparams(const nnpgpu_ctx* ctx, int type);
/* the networks' parameters in the same order, to read and to replace (a trainer's update; later
 * evaluations use them; refused with NNPGPU_ERR_BUSY while serving), and the potential with its
 * current parameters written in the reference's text format (NNP::write, src/nnp/nnp.cpp:198-237).
 * Without a device (nnpgpu_create returned NNPGPU_ERR_CUDA but a context) they act on the parsed
 * potential alone. */
int nnpgpu_get_params(const nnpgpu_ctx* ctx, int type, double* params);
int nnpgpu_set_params(nnpgpu_ctx* ctx, int type, const double* params);
int nnpgpu_write_potential(nnpgpu_ctx* ctx, const char* path);
/* ---- training with forces: the force trainer's loss (NNPTEF::error, src/nnp/nnptef.cpp:1043-1135)
 *   sum_s loss(dE_s) + sum over atoms 0.5 beta |(F - F_ref)/N_s|^2,
 * F the forces of NNP::force (minimum-image rule), E without vacuum energies, loss and delta as
 * for nnpgpu_train_grad; force_ref[sum(natoms)*3].  grad is the exact gradient of that loss (the
 * reference's nnptef.cpp keeps only each atom's own terms and calls BasisR::rho, which this
 * snapshot does not define); error[0] = the loss, error[1] = sum of dE^2, error[2] = sum over
 * atoms of |(F - F_ref)/N_s|^2.  FP32 descriptors, networks and second derivatives, FP64 sums. */
int nnpgpu_train_force_grad(nnpgpu_ctx* ctx, int nstruc, const int* natoms, const double* posn, const int* species,
                            const double* cell, const double* energy_ref, const double* force_ref, double beta, int loss,
                            double delta, double* error, double* grad);
int nnpgpu_train_grad(nnpgpu_ctx* ctx, int nstruc, const int* natoms, const double* posn, const int* species,
                      const double* cell, const double* energy_ref, int loss, double delta, double* error, double* grad);

/* ---- launch-shape autotuner (no counterpart in the reference, which has no launch shapes).
 * Times the batched path on the given batch (host buffers, as nnpgpu_compute) for each candidate
 * of each knob - centre atoms (warps) per CTA of the neighbour, descriptor and chain-rule kernels
 * (1, 2, 4) and the atom tile of the FP32 networks (16, 32, 64; skipped with NNPGPU_BF16) - one
 * knob at a time, from stage events inside the captured launch sequence, and keeps the fastest.
 * flags: NNPGPU_BF16, NNPGPU_FORCE (the chain-rule knob is tuned only with it).  report (may be
 * NULL) receives the per-candidate times.  Later calls of the context use the chosen shapes;
 * nnpgpu_get_tune / nnpgpu_set_tune read and restore them (e.g. from a caller's cache). */
int nnpgpu_autotune(nnpgpu_ctx* ctx, int nstruc, const int* natoms, const double* posn, const int* species,
                    const double* cell, int flags, char* report, int report_len);
int nnpgpu_get_tune(const nnpgpu_ctx* ctx, int* warps_nbr, int* warps_symm, int* warps_force, int* nn_tile);
int nnpgpu_set_tune(nnpgpu_ctx* ctx, int warps_nbr, int warps_symm, int warps_force, int nn_tile);

/* ---- failure detection (no counterpart in the reference, which has no device waits).  Bound on
 * each mbarrier wait of the tensor-core network kernel (NNPGPU_BF16), in polls; the default
 * 4194304 is about half a second.  A wait that runs out ends the call with NNPGPU_ERR_TIMEOUT after
 * the kernel has waited (bounded) for the copies and MMAs it issued and freed its TMEM, so the
 * context stays usable; if those did not finish either the message says to destroy the context.
 * 0 makes every wait give up at once (a test of this path). */
int nnpgpu_set_wait_limit(nnpgpu_ctx* ctx, int polls);

/* ---- serving: continuous batching of energy+force requests (no counterpart in the
 * reference, whose compute tool evaluates a fixed file list; it serves the same call as
 * nnpgpu_compute for requests that arrive over time). */
typedef struct nnpgpu_serve_opts {
  int max_batch_atoms;     /* atoms admitted into one device batch (0 = automatic) */
  int max_inflight;        /* batches in flight on the device (>= 1) */
  size_t hbm_budget_bytes; /* admission budget for resident state + batch buffers (0 = context budget) */
  double skin;             /* neighbour-list skin for resident structures, Angstrom (0 = rebuild always) */
  int flags;               /* NNPGPU_BF16 etc. applied to every request */
} nnpgpu_serve_opts;

int nnpgpu_serve_start(nnpgpu_ctx* ctx, const nnpgpu_serve_opts* opts);
/* Copies the request; resident_key >= 0 keeps the structure's state on the device between
 * requests with the same key (MD-style repeat steps), -1 for a one-off request. */
int nnpgpu_submit(nnpgpu_ctx* ctx, int natoms, const double* posn, const int* species, const double* cell,
                  long long resident_key, long long* request_id);
/* NNPGPU_OK when done (results copied out, request released), NNPGPU_ERR_BUSY when not yet. */
int nnpgpu_poll(nnpgpu_ctx* ctx, long long request_id, double* energy, double* force, double* latency_s);
int nnpgpu_serve_stop(nnpgpu_ctx* ctx);

/* ---- molecular dynamics on resident device state.  Replaces the reference's MD job
 * (src/torch/torch.cpp:267-275): velocity-Verlet steps (Verlet::compute,
 * src/torch/integrator.cpp:170-193) around Engine::compute (src/torch/engine.cpp:107-118) with the
 * NNP potential PotNNPE::compute (src/torch/pot_nnpe.cpp:175-295: energy including the species
 * vacuum energies, forces with NNP::force's minimum-image rule).  Positions, velocities, forces
 * and masses stay on the GPU.  Units as the reference: v += (dt/2) F/m with F in the potential's
 * force unit and mass in whatever unit the caller pairs with dt (no conversion).  The first step
 * starts from zero forces, as the reference's MD job does; call nnpgpu_md_forces first for a
 * step that starts from the forces at the initial positions.
 * Neighbour lists: a list at rc + skin stays resident and is refreshed exactly at rc every step
 * (each step's forces equal a fresh list's), rebuilt when an atom has moved more than skin/2;
 * skin = 0, or a cell with several images of an atom within rc, rebuilds every step.
 *   posn, vel (may be NULL = zero) natoms*3; species natoms; mass natoms (per atom, > 0);
 *   cell 9 (column-major lattice vectors); flags: NNPGPU_BF16 or 0. */
typedef struct nnpgpu_md nnpgpu_md;
int nnpgpu_md_create(nnpgpu_ctx* ctx, int natoms, const double* posn, const double* vel, const int* species,
                     const double* mass, const double* cell, double dt, double skin, int flags, nnpgpu_md** out);
/* forces and potential energy at the current positions (no step) */
int nnpgpu_md_forces(nnpgpu_md* md, double* pe);
/* nsteps velocity-Verlet steps; pe[t], ke[t] (may be NULL) receive each step's potential energy
 * and kinetic energy 0.5 sum m |v|^2 */
int nnpgpu_md_run(nnpgpu_md* md, int nsteps, double* pe, double* ke);
/* positions (wrapped into the cell as Cell::returnToCell, src/struc/cell.cpp:84-94), velocities,
 * forces (each may be NULL) and the number of resident-list builds so far */
int nnpgpu_md_state(nnpgpu_md* md, double* posn, double* vel, double* force, int* rebuilds);
void nnpgpu_md_destroy(nnpgpu_md* md);

#ifdef __cplusplus
}
#endif
#endif
