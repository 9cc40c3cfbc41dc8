/*
 * mdg.h -- C ABI of libmdg, the GB300 (sm_103a) force-and-step engine behind
 * the mdpy constraint / ensemble / integrator API.
 *
 * The reference (mdpy v0.2.1) is pure Python and has no FFI; each entry point
 * below names the reference interface whose work it takes over (paths are
 * relative to the mdpy source tree).  The Python host layer in
 * mdpy_gb300/ binds these through ctypes.
 *
 * Conventions
 *  - Every function returns an int status: MDG_OK (0) or an MDG_ERR_* code.
 *    mdg_last_error() returns a message for the calling thread's last error.
 *  - Units are mdpy's: Angstrom, Dalton, femtosecond, elementary charge,
 *    energy Da*A^2/fs^2 (mdpy/unit/__init__.py:31-49).
 *  - Boxes are orthorhombic (the diagonal of mdpy's pbc_matrix); a
 *    non-diagonal pbc_matrix is rejected with MDG_ERR_BOX.
 *  - Arrays are row-major.  Host pointers are read/written synchronously
 *    unless a function says `where`; with where == MDG_DEVICE the pointer is a
 *    device address (e.g. a torch tensor's data_ptr()) in the system's device.
 *  - The library owns all device memory of a system; nothing is kept from a
 *    caller's pointer after the call returns.
 *  - Calls on one system are not thread-safe; use one system per thread.
 *  - Work is issued on the system's stream (mdg_system_set_stream).
 */
#ifndef MDG_H
#define MDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDG_API __attribute__((visibility("default")))

/* status codes */
#define MDG_OK 0
#define MDG_ERR_INVALID 1       /* bad argument or call order */
#define MDG_ERR_CUDA 2          /* CUDA runtime failure */
#define MDG_ERR_NOMEM 3         /* device allocation failed */
#define MDG_ERR_BOX 4           /* box not orthorhombic / not positive */
#define MDG_ERR_CUTOFF 5        /* cutoff >= half the box (minimum image breaks) */
#define MDG_ERR_PARTICLE_LOSS 6 /* non-finite position or velocity, or a position
                                   two or more box lengths from the central image */
#define MDG_ERR_OVERFLOW 7      /* fixed-point force/energy overflow */
#define MDG_ERR_CUFFT 8         /* cuFFT failure */
#define MDG_ERR_TIMEOUT 9       /* a bounded device wait gave up */
#define MDG_ERR_CAPACITY 10     /* caller buffer too small */
#define MDG_ERR_STATE 11        /* operation needs state that is not set */

/* memory location of a caller pointer */
#define MDG_HOST 0
#define MDG_DEVICE 1

/* force / energy terms (bit masks and energy slots) */
#define MDG_TERM_LJ 0          /* Lennard-Jones (incl. 1-4 pairs)            */
#define MDG_TERM_COUL_REAL 1   /* Ewald real space erfc, or bare Coulomb     */
#define MDG_TERM_COUL_RECIP 2  /* PME reciprocal + self + net-charge + excl. */
#define MDG_TERM_BOND 3
#define MDG_TERM_ANGLE 4
#define MDG_TERM_DIHEDRAL 5
#define MDG_TERM_IMPROPER 6
#define MDG_NUM_TERMS 7
#define MDG_MASK(t) (1u << (t))
#define MDG_MASK_ALL ((1u << MDG_NUM_TERMS) - 1u)

/* Coulomb modes of the short-range constraint */
#define MDG_COUL_NONE 0
#define MDG_COUL_EWALD 1 /* erfc(beta r)/r inside the cutoff            */
#define MDG_COUL_BARE 2  /* 1/r, all pairs, minimum image, no cutoff   */

/* integrators */
#define MDG_INTEGRATOR_VERLET 0
#define MDG_INTEGRATOR_LANGEVIN 1

typedef struct mdg_system mdg_system;

/* ---- diagnostics -------------------------------------------------------- */
MDG_API int mdg_version(int *major, int *minor);
MDG_API const char *mdg_last_error(void);

/* ---- system lifetime ---------------------------------------------------- */
/* Replaces the device state the reference rebuilds per call
 * (Ensemble.__init__ + State, mdpy/ensemble.py:16-31, mdpy/core/state.py:19-28):
 * allocates a system of n_atoms on `device` with box edges box[3]. */
MDG_API int mdg_system_create(int device, int n_atoms, const double *box, mdg_system **out);
MDG_API int mdg_system_destroy(mdg_system *sys);
/* cudaStream_t passed as void*; NULL restores the system's own stream */
MDG_API int mdg_system_set_stream(mdg_system *sys, void *stream);
/* State.set_pbc_matrix (mdpy/core/state.py:47-54), diagonal only; in a batch
 * every system gets this box */
MDG_API int mdg_system_set_box(mdg_system *sys, const double *box);

/* ---- batches of independent systems (no reference counterpart: mdpy runs
 * one Ensemble per process; a batch runs many small ensembles in one set of
 * launches).  System q owns atoms [off_q, off_q + n_atoms[q]) of every per-atom
 * array (off_q = sum of the earlier counts); it has its own box (boxes[3q..3q+2]),
 * PME grid and energies; nonbonded, PME order/beta and integrator settings are
 * shared.  Exclusion partners and bonded terms must stay inside one system.
 * Forces, energies and trajectories of each system are those it would have
 * alone, up to float rounding of the batched FFT.  A single system is a batch
 * of one. */
MDG_API int mdg_system_create_batch(int device, int n_systems, const int *n_atoms,
                                    const double *boxes, mdg_system **out);
MDG_API int mdg_num_systems(mdg_system *sys, int *n_systems);
/* boxes (n_systems, 3) */
MDG_API int mdg_system_set_boxes(mdg_system *sys, const double *boxes);
/* PME with one grid per system: grids (n_systems, 3); systems with equal grids
 * share one batched FFT */
MDG_API int mdg_pme_config_batch(mdg_system *sys, const int *grids, int order, double beta);
/* energies (n_systems, MDG_NUM_TERMS) and kinetic (n_systems) of the last
 * evaluation, per system; either may be NULL */
MDG_API int mdg_get_energies_batch(mdg_system *sys, double *energies, double *kinetic);

/* ---- static parameters (bind_ensemble work) ----------------------------- */
/* Topology.join masses/charges (mdpy/core/topology.py:59-70) */
MDG_API int mdg_set_masses(mdg_system *sys, const double *masses);
MDG_API int mdg_set_charges(mdg_system *sys, const double *charges);
/* CharmmNonbondedConstraint.bind_ensemble per-atom [eps, sigma, eps14, sigma14]
 * (mdpy/constraint/charmm_nonbonded_constraint.py:48-62), shape (n, 4) */
MDG_API int mdg_set_lj(mdg_system *sys, const double *params);
/* Topology.bonded_particles (1-2/1-3, excluded) and scaling_particles (1-4)
 * as dense -1 padded (n, width) arrays (mdpy/core/topology.py:71-79) */
MDG_API int mdg_set_exclusions(mdg_system *sys, const int32_t *bonded, int bonded_width,
                               const int32_t *scaling, int scaling_width);

/* ---- nonbonded configuration ------------------------------------------- */
/* CharmmNonbondedConstraint(cutoff_radius) + ElectrostaticConstraint, re-designed:
 * LJ on/off, optional CHARMM switch from `switch_radius` (<= 0: hard cutoff as
 * the reference), Coulomb mode MDG_COUL_*, Ewald splitting `beta` (1/A). */
MDG_API int mdg_nonbonded_config(mdg_system *sys, double cutoff, double switch_radius,
                                 int lj_on, int coulomb_mode, double beta);
/* PME reciprocal space (no reference counterpart; LONG_RANGE_SOLVER names it,
 * mdpy/constraint/__init__.py:22): grid K[3], B-spline order, splitting beta. */
MDG_API int mdg_pme_config(mdg_system *sys, const int *grid, int order, double beta);
/* spatial re-sort interval (steps) of the atom clusters; default 20 */
MDG_API int mdg_set_reorder_interval(mdg_system *sys, int steps);

/* ---- bonded terms (CharmmBond/Angle/Dihedral/ImproperConstraint.bind_ensemble) */
/* bonds: idx (n,2), prm (n,2) = (k, r0)          charmm_bond_constraint.py:32-50
 * angles: idx (n,3), prm (n,4) = (k, th0, ku, u0) charmm_angle_constraint.py:116-136
 * dihedrals: idx (n,4), prm (n,3) = (k, n, delta) charmm_dihedral_constraint.py:33-56
 * impropers: idx (n,4), prm (n,2) = (k, psi0)     charmm_improper_constraint.py  */
MDG_API int mdg_set_bonds(mdg_system *sys, int n, const int32_t *idx, const double *prm);
MDG_API int mdg_set_angles(mdg_system *sys, int n, const int32_t *idx, const double *prm);
MDG_API int mdg_set_dihedrals(mdg_system *sys, int n, const int32_t *idx, const double *prm);
MDG_API int mdg_set_impropers(mdg_system *sys, int n, const int32_t *idx, const double *prm);

/* ---- state ------------------------------------------------------------- */
/* State.set_positions / set_velocities (mdpy/core/state.py:56-65), (n,3) FP64 */
MDG_API int mdg_set_positions(mdg_system *sys, const double *x, int where);
MDG_API int mdg_set_velocities(mdg_system *sys, const double *v, int where);
/* positions wrapped into [-L/2, L/2) as wrap_positions (mdpy/utils/pbc.py:28-36) */
MDG_API int mdg_get_positions(mdg_system *sys, double *x, int where);
MDG_API int mdg_get_velocities(mdg_system *sys, double *v, int where);

/* ---- forces and energies ----------------------------------------------- */
/* Ensemble.update / Constraint.update (mdpy/ensemble.py:53-61): evaluate the
 * terms in `mask` into the system force buffer (int64 fixed point, 2^-32)
 * and their energies. */
MDG_API int mdg_compute_forces(mdg_system *sys, unsigned mask);
/* Ensemble.forces / Constraint.forces: (n,3) FP64 in atom order */
MDG_API int mdg_get_forces(mdg_system *sys, double *f, int where);
/* energies[MDG_NUM_TERMS] of the last evaluation (reciprocal slot includes the
 * self, net-charge and exclusion terms) and the kinetic energy; a batch
 * reports the sums over its systems */
MDG_API int mdg_get_energies(mdg_system *sys, double *energies, double *kinetic);
/* Ensemble._update_kinetic_energy (mdpy/ensemble.py:63-71), FP64 */
MDG_API int mdg_kinetic_energy(mdg_system *sys, double *kinetic);

/* Energy snapshots for log dumping without a host synchronisation per dump:
 * the device->host half of LogDumper.dump (mdpy/dumper/log_dumper.py:
 * 105-208, which reads Ensemble energies as Simulation.integrate reaches
 * each dump step, mdpy/simulation.py:60-70).  mdg_energy_snapshot enqueues
 * on the system's stream a copy of the energy words of the last evaluation
 * with energies (and of the device status word) into pinned ring slot `slot`
 * (0 <= slot < MDG_SNAPSHOT_SLOTS, allocated on first use) and records an
 * event; it returns without waiting, so the steps enqueued after it keep the
 * GPU busy while the host formats earlier rows.  mdg_energy_snapshot_read
 * turns slot `slot` into energies[MDG_NUM_TERMS] and *kinetic exactly as
 * mdg_get_energies would have at the snapshot: with wait != 0 it waits for
 * the copy; with wait == 0 it sets *ready = 0 and leaves the outputs alone
 * if the copy has not completed yet (*ready = 1 otherwise; ready may be
 * NULL when wait != 0).  A device error raised before the snapshot (particle
 * loss, fixed-point overflow) is returned by the read.  Reusing a slot
 * before its read overwrites it. */
#define MDG_SNAPSHOT_SLOTS 8
MDG_API int mdg_energy_snapshot(mdg_system *sys, int slot);
MDG_API int mdg_energy_snapshot_read(mdg_system *sys, int slot, int wait, double *energies,
                                     double *kinetic, int *ready);

/* One call for a host-driven loop (no reference counterpart; it bundles
 * State.set_positions/set_velocities, Integrator.integrate and the reads of
 * State.positions/velocities and the energies): copies x_in / v_in (host,
 * (n,3); NULL = keep the device state) to the device, runs n_steps steps of
 * the configured integrator on the terms in `mask`, copies the wrapped
 * positions, the velocities (host (n,3); NULL = skip) and the energies
 * (energies[MDG_NUM_TERMS], *kinetic; NULL = skip) back, all on the system's
 * stream with one synchronisation at the end.  Incoming positions are
 * compared on the device with the state as it would be reported (one more
 * synchronisation): equal ones -- the previous call's outputs fed back --
 * keep the forces already computed for them and the cluster order; others
 * start with a re-sort and a fresh force evaluation, as mdg_set_positions
 * does. */
MDG_API int mdg_step_host(mdg_system *sys, const double *x_in, const double *v_in, int n_steps,
                          unsigned mask, double *x_out, double *v_out, double *energies,
                          double *kinetic);

/* ---- launch shapes and the autotuner (no reference counterpart) ---------
 * A launch shape is MDG_SHAPE_FIELDS ints:
 *   [MDG_SHAPE_SPLIT]          work items (one warp each) per 32-atom cluster in
 *                              the pair kernel: 1, 2, 4, 8, 16 (default 4);
 *   [MDG_SHAPE_PERSISTENT]     0 = one CTA per work item; n = n resident CTAs
 *                              per SM (1..24) pulling work items from a device
 *                              counter (default 0);
 *   [MDG_SHAPE_PME_BLOCK]      threads per block of PME spread/gather: 64, 128,
 *                              256 (default 256);
 *   [MDG_SHAPE_SIDE_PRIORITY]  1 runs PME, special pairs and bonded terms on
 *                              highest-priority streams beside the pair kernel
 *                              (default 0);
 *   [MDG_SHAPE_SPLIT_RINGS]    1 sweeps j atoms without LJ parameters in chunks
 *                              that skip the LJ arithmetic (default 1);
 *   [MDG_SHAPE_PME_TILES]      bit 0: spreading through a shared-memory tile of
 *                              the block's grid patch, bit 1: gathering from one
 *                              (default 0);
 *   [MDG_SHAPE_HALF]           1: each half warp sweeps its own j list against 16
 *                              i atoms (j atoms within rc of those 16 only); 2:
 *                              each quarter warp against 8 i atoms; 0: one list
 *                              against all 32 (default 0).
 * Results depend on the shape only through float rounding of partial sums
 * (the PME grid and tiling change nothing: int64 sums); for a fixed shape
 * they are bit-reproducible. */
#define MDG_SHAPE_SPLIT 0
#define MDG_SHAPE_PERSISTENT 1
#define MDG_SHAPE_PME_BLOCK 2
#define MDG_SHAPE_SIDE_PRIORITY 3
#define MDG_SHAPE_SPLIT_RINGS 4
#define MDG_SHAPE_PME_TILES 5
#define MDG_SHAPE_HALF 6
#define MDG_SHAPE_FIELDS 7
MDG_API int mdg_set_launch_shape(mdg_system *sys, const int *shape);
MDG_API int mdg_get_launch_shape(mdg_system *sys, int *shape);
/* Picks the fastest launch shape: with an integrator configured it times MD
 * steps as mdg_integrate runs them (captured single-step graphs replayed from
 * a saved state, which is restored afterwards), else force evaluations of
 * `mask`.  Phase one varies the pair kernel (split 2/4/8 x persistent 0/20/24
 * x split rings 0/1 x half 0/1/2), phase two PME and the streams (block 64/128/256 x tiles
 * 0-3 x side priority 0/1) around phase one's best; then the four fastest and
 * the shape in use are re-timed, interleaved, over 4 x reps and the fastest
 * is kept; *best_ms (may be NULL) receives its time.  Leaves no valid force
 * evaluation. */
MDG_API int mdg_autotune(mdg_system *sys, unsigned mask, int reps, double *best_ms);

/* ---- energy minimisation ------------------------------------------------ */
/* One move of SteepestDescentMinimizer.minimize
 * (mdpy/minimizer/steepest_descent_minimizer.py:39-42): x_i += alpha F_i/|F_i|
 * from the forces of the last evaluation (atoms with zero force stay put).
 * The caller re-evaluates (mdg_compute_forces) and tests the energy. */
MDG_API int mdg_minimize_step(mdg_system *sys, double alpha);

/* ---- no-allocation entry point (no reference counterpart) --------------
 * For callers that must not have device memory allocated behind their
 * back: a host program whose own pool already owns the GPU's memory (it
 * reserves it up front and hands out every buffer itself, so a library
 * cudaMalloc either fails or breaks its accounting), or a tight loop that
 * cannot afford cudaMalloc/cudaFree, which may synchronise the whole device
 * and stall every other stream.
 * kinetic[n_systems] (host) = each system's kinetic energy, bit for bit the
 * per-system values mdg_kinetic_energy produces (mdg_get_energies_batch),
 * computed without allocating device memory: the int64 accumulators live in
 * a static device array sized for MDG_NOALLOC_MAX_SYSTEMS systems (128 KiB,
 * held by every GPU that loads the library until the process exits),
 * zeroed by each call; a larger batch fails with MDG_ERR_INVALID.  The first
 * call on a device looks the array's address up (cudaGetSymbolAddress) and
 * must come before any stream capture.  All calls share the array: calls
 * that overlap in time (other host threads, or other streams whose work
 * overlaps) race on it. */
#define MDG_NOALLOC_MAX_SYSTEMS 1024
MDG_API int mdg_kinetic_energies_noalloc(mdg_system *sys, double *kinetic);

/* ---- integration ------------------------------------------------------- */
/* Multiple time steps (no reference counterpart): with k > 1 the
 * reciprocal-space force (PME and the excluded-pair correction) enters only
 * the evaluation that ends every k-th step, weighted by k, and is left out of
 * the others -- the impulse (Verlet-I / r-RESPA) scheme with an outer step of
 * k dt; the other terms are evaluated every step.  Energies stay complete
 * (the reciprocal energy is computed on energy steps whatever the phase);
 * mdg_get_forces after mdg_integrate returns the weighted buffer.  k = 1
 * (default) is the ordinary integrator. */
MDG_API int mdg_set_mts(mdg_system *sys, int k);

/* ---- learned slow force (no reference counterpart) ----------------------
 * The multiple-time-step form with a learned prediction between full PME
 * evaluations.  The slow force (PME plus the excluded-pair correction) is
 * computed in full at every k-th step; in between it is predicted as
 * F_slow(t0) + J (x(t) - x(t0)) + G(x(t)) - G(x(t0)), t0 the last full
 * evaluation, J the field-gradient term (mdg_learned_set_terms) and G a
 * rotation-equivariant network: per atom 64 invariant radial features of the
 * neighbours within rf (sum_j q_j phi_b(r_ij) and sum_j phi_b(r_ij) over 32
 * cubic B-spline bins), a BF16 MLP 64-128-128-16 (SiLU, FP32 accumulation)
 * and G_i = sum_b C_ib q_i sum_j q_j psi_b(r_ij) (x_i - x_j) / rf^2 over 16
 * radial functions psi_b.  Each full evaluation judges the prediction made
 * for it (RMS error over RMS total force); above the threshold the next
 * interval uses the impulse scheme of mdg_set_mts instead.  One system only.
 *
 * mdg_learned_config allocates the network's buffers: feature radius rf (A),
 * neighbour-list skin (A), list entries per atom.  Parameters are one FP32
 * vector of mdg_learned_num_params entries: feature shift [64], feature
 * inverse scale [64], W1 [64][128], b1 [128], W2 [128][128], b2 [128],
 * W3 [128][16], b3 [16], output scale [1] (weights [in][out]). */
MDG_API int mdg_learned_config(mdg_system *sys, double rf, double skin, int list_capacity);
MDG_API int mdg_learned_num_params(int32_t *n);
MDG_API int mdg_learned_set_params(mdg_system *sys, const float *params, int32_t n);
MDG_API int mdg_learned_get_params(mdg_system *sys, float *params, int32_t n);
/* Training.  mdg_learned_frame(slot) evaluates the slow force at the current
 * positions and runs the network forward, keeping what the backward pass
 * needs (slots 0 and 1: two frames a few steps apart of a plain run);
 * mdg_learned_frame_data copies a frame's raw features (n x 64), vector
 * basis (n x 48, index 3 b + axis), slow force (n x 3) and prediction G
 * (n x 3) to the host (any pointer may be null).  mdg_learned_train_step
 * fits G(x1) - G(x0) to F_slow(x1) - F_slow(x0) over the two frames: loss =
 * sum |residual|^2 / sum |F_slow(x1) - F_slow(x0)|^2 of the frames before
 * the update (1 = no better than holding the slow force), one Adam step
 * (beta 0.9 / 0.999, step number t >= 1, rate lr). */
MDG_API int mdg_learned_frame(mdg_system *sys, int32_t slot);
MDG_API int mdg_learned_frame_data(mdg_system *sys, int32_t slot, float *features, float *vectors,
                                   float *slow_force, float *predicted);
MDG_API int mdg_learned_train_step(mdg_system *sys, float lr, int32_t t, double *loss);
/* the inference kernel (mdg_learned_set_kernel) on the features of a frame;
 * G (n x 3) to the host when `predicted` is not null */
MDG_API int mdg_learned_predict(mdg_system *sys, int32_t slot, float *predicted);
/* k >= 2: use the learned form with outer step k and judge threshold;
 * k = 0 or 1: off (and the impulse scheme off).  mdg_set_mts turns it off. */
MDG_API int mdg_set_mts_learned(mdg_system *sys, int32_t k, double threshold);
/* Terms of the prediction between full evaluations (default: the network
 * alone -- on flexible water the field-gradient term removes only ~4 % of
 * the held force's error at k = 4: the slow force changes mostly through
 * the motion of the other atoms):
 * field_gradient: J_i (x_i(t) - x_i(t0)) with J_i = d F_slow,i / d x_i at t0
 * (the other atoms held), from the B-spline second derivatives of the PME
 * potential (order 4) less the atom's own smeared charge and its excluded
 * partners; network: G(x(t)) - G(x(t0)), trained on what the first term
 * leaves.  Both off: the slow force of t0 is held. */
MDG_API int mdg_learned_set_terms(mdg_system *sys, int32_t field_gradient, int32_t network);
/* 1: the tcgen05 tensor-core MLP kernel for inference; 0: the SIMT kernel */
MDG_API int mdg_learned_set_kernel(mdg_system *sys, int32_t tensor_cores);
/* Test of the tcgen05 inference kernel's bounded waits (no reference
 * counterpart).  Arms a one-shot test: the next launch of that kernel
 * withholds its first bulk copy (weights and first feature tile), so its
 * first mbarrier wait gives up after 10 ms of wall time instead of the
 * usual 1 s.  The kernel then raises MDG_ERR_TIMEOUT, has no MMA and no copy
 * in flight to wait for, frees its tensor memory and returns; the call that
 * launched it (e.g. mdg_learned_predict) returns MDG_ERR_TIMEOUT and the
 * system stays usable.  MDG_ERR_STATE unless the tensor-core kernel is
 * selected. */
MDG_API int mdg_learned_wait_test(mdg_system *sys);
/* out[8]: last judged error, largest, sum of errors, judgements, fallbacks,
 * last training loss, last training target norm, mode of the current
 * interval (0 learned, 1 impulse fallback) */
MDG_API int mdg_learned_stats(mdg_system *sys, double *out8);
MDG_API int mdg_learned_reset_stats(mdg_system *sys);
/* VerletIntegrator / LangevinIntegrator (mdpy/integrator/*.py) re-designed:
 * velocity Verlet or Groenbech-Jensen--Farago Langevin, FP64 x/v, one force
 * evaluation per step, Philox4x32-10 noise keyed by (seed, atom, step). */
MDG_API int mdg_integrator_config(mdg_system *sys, int kind, double dt, double temperature,
                                  double friction, uint64_t seed);
/* Integrator.integrate(ensemble, num_steps) (mdpy/integrator/integrator.py:24-27):
 * advances n_steps over the force terms in `mask`; energies of the final
 * step are evaluated when want_energy != 0.  Steps run as CUDA graphs. */
MDG_API int mdg_integrate(mdg_system *sys, int n_steps, unsigned mask, int want_energy);
/* current step counter (the Philox counter of the next step) */
MDG_API int mdg_get_step(mdg_system *sys, uint64_t *step);
MDG_API int mdg_set_step(mdg_system *sys, uint64_t step);

/* ---- parity / diagnostics ---------------------------------------------- */
/* All unordered pairs (atom indices i<j, int32 pairs) that the short-range
 * kernel evaluates with r <= cutoff, from the same kernel code path as the
 * forces.  *count receives the total; at most `capacity` pairs are written. */
MDG_API int mdg_pairset_dump(mdg_system *sys, int32_t *pairs, int64_t capacity,
                             int64_t *count);
/* thermostat noise of step `step`, (n,3) float32 (same Philox stream as the
 * Langevin kernel) */
MDG_API int mdg_langevin_noise(mdg_system *sys, uint64_t step, float *out);
/* device-side status word: 0 or MDG_ERR_* raised by a kernel since the last call */
MDG_API int mdg_check_status(mdg_system *sys);
/* statistics of the last nonbonded evaluation: [0] pair evaluations issued,
 * [1] pairs inside the cutoff, [2] cluster candidates, [3] clusters */
MDG_API int mdg_nonbonded_stats(mdg_system *sys, int64_t *stats);
/* number of kernels libmdg has launched on this system so far */
MDG_API int mdg_launch_count(mdg_system *sys, int64_t *count);

/* graph granularity of mdg_integrate: MDG_GRAPH_CHUNK (default) replays
 * `reorder_interval` steps per graph launch; MDG_GRAPH_STEP replays one graph
 * per MD step (so a caller can bracket single steps with events). */
#define MDG_GRAPH_CHUNK 0
#define MDG_GRAPH_STEP 1
MDG_API int mdg_set_graph_mode(mdg_system *sys, int mode);

/* Launch one stage of a force evaluation on the system stream, for timing and
 * profiling (the state must have been evaluated once).  Stages that
 * accumulate forces leave the force buffer invalid. */
#define MDG_STAGE_PACK 0
#define MDG_STAGE_NONBONDED 1
#define MDG_STAGE_SPECIAL 2
#define MDG_STAGE_PME 3
#define MDG_STAGE_BONDED 4
#define MDG_STAGE_REORDER 5
#define MDG_STAGE_INTEGRATE 6 /* pre + post update kernels */
#define MDG_STAGE_NONBONDED_ENERGY 7 /* the pair kernel's variant that also sums energies */
MDG_API int mdg_launch_stage(mdg_system *sys, int stage, unsigned mask);

#ifdef __cplusplus
}
#endif
#endif /* MDG_H */
