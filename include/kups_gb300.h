/*
 * kups_gb300 — C ABI of the GB300 (sm_103a) particle-interaction kernels.
 *
 * Conventions shared by every entry point:
 *   - all array pointers are DEVICE pointers owned by the caller; nothing is
 *     allocated or freed by the library (scratch space is passed in as
 *     `workspace`, sized by the matching *_workspace_bytes query, except in
 *     kups_ewald_recip_static, which uses a fixed array of the library);
 *   - `stream` is a cudaStream_t passed as void*; every call is stream-ordered
 *     and never synchronises the device; every call except
 *     kups_ewald_recip_static is safe to capture in a CUDA graph (it issues
 *     only kernel launches and cudaMemsetAsync);
 *   - a workspace holds nothing a later call needs, except the fused MD's
 *     (kups_lj_md_run), whose per-system records let the next call on the
 *     same workspace resume its Verlet lists (kups_md_args.reuse_lists);
 *   - the return value reports host-side validation and launch errors
 *     (KUPS_OK, KUPS_ERR_INVALID, KUPS_ERR_CUDA; kups_ewald_recip_static also
 *     returns KUPS_ERR_CAPACITY and KUPS_ERR_UNSUPPORTED, see there); device-side conditions
 *     (capacity overflow, non-finite input) are written to the caller's
 *     device `kups_status`, which the caller reads back with its outputs.
 *     Kernels never trap and never write past a capacity: on overflow they
 *     record the capacity that would have sufficed in `required`, which is
 *     how kUPS's Capacity / propagate_and_fix grow-and-retry loop
 *     (src/kups/core/capacity.py:48-133, src/kups/core/propagator.py:137-172)
 *     maps onto this library.
 *   - unit cells are lower-triangular, given by `tril` = [L00, L10, L11, L20,
 *     L21, L22] per system, row convention r = f @ L
 *     (src/kups/core/unitcell.py:251-300).
 */
#ifndef KUPS_GB300_H
#define KUPS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kups_status {
  int32_t code;      /* KUPS_OK or a KUPS_ERR_* code */
  int32_t detail;    /* KUPS_CAP_* for capacity errors */
  int64_t required;  /* capacity that would have sufficed */
  int64_t first_bad; /* first offending particle / system index, -1 if none */
} kups_status;

enum {
  KUPS_OK = 0,
  KUPS_ERR_CAPACITY = 1,
  KUPS_ERR_NONFINITE = 2,
  KUPS_ERR_INVALID = 3,
  KUPS_ERR_CUDA = 4,
  KUPS_ERR_UNSUPPORTED = 5
};

enum {
  KUPS_CAP_EDGES = 1,     /* edge buffer of the neighbour list */
  KUPS_CAP_NEIGHBORS = 2, /* per-atom Verlet-list slots of the fused MD kernel */
  KUPS_CAP_GHOSTS = 3,    /* periodic-image copies held in shared memory */
  KUPS_CAP_CELLS = 4,     /* cells of the per-system cell grid */
  KUPS_CAP_ATOMS = 5      /* atoms of one system held in shared memory */
};

const char *kups_version(void);
const char *kups_error_string(int32_t code);

/* ------------------------------------------------------------------------
 * Neighbour list — replaces CellListNeighborList.__call__ and
 * DenseNearestNeighborList.__call__ (src/kups/core/neighborlist.py:985-1077,
 * 902-982; protocol NearestNeighborList.__call__ :226-255, rh = None).
 *
 * Produces the directed edge set of basic_neighborlist (:743-786): pairs of
 * the same system and valid inclusion segment with |x_j - x_i + s @ L| < rc
 * (strict, float64), the periodic-image path of
 * _apply_distance_cutoff_w_images (:595-624) when 2 rc exceeds a cell width,
 * and the minimum-image-only exclusion rule (:731-735).  Edges are grouped by
 * i (lh) in increasing order; entries [n_edges, edge_capacity) are padded
 * with i = j = n_particles and a zero shift, as _compact_edges pads (:651-689).
 * A system whose cutoff needs more than 1331 image offsets per pair (a cutoff
 * of about five cell widths) gets no edges and KUPS_ERR_UNSUPPORTED is recorded
 * with its index; an infinite cutoff means the minimum image only.
 *
 *   positions  f64 [n_particles, 3]   Cartesian
 *   system     i32 [n_particles]      values outside [0, n_systems) = empty slot
 *   inclusion  i32 [n_particles]      valid iff in [0, n_inclusion)
 *   exclusion  i32 [n_particles]
 *   tril       f64 [n_systems, 6],  cutoffs f64 [n_systems]
 *   edges      i32 [edge_capacity, 2],  shifts i32 [edge_capacity, 3]
 *   n_edges    i64 [1]  (device) number of edges found (may exceed capacity)
 * ------------------------------------------------------------------------ */
size_t kups_neighborlist_workspace_bytes(int64_t n_particles, int32_t n_systems);
int32_t kups_neighborlist_build(const double *positions, const int32_t *system,
                                const int32_t *inclusion, const int32_t *exclusion,
                                int64_t n_particles, int32_t n_inclusion,
                                const double *tril, const double *cutoffs,
                                int32_t n_systems, int32_t *edges, int32_t *shifts,
                                int64_t edge_capacity, int64_t *n_edges,
                                void *workspace, size_t workspace_bytes,
                                kups_status *status, void *stream);

/* kups_neighborlist_build_rh replaces NearestNeighborList.__call__ with a
 * separate rh table (src/kups/core/neighborlist.py:226-255, basic_neighborlist
 * :743-786): directed edges (i in lh, j in rh) of the same system and inclusion
 * label within the system's cutoff, under the image rule of the full mode with
 * the difference lh - rh, the exclusion labels of lh and rh dropping only the
 * minimum image (:731-735).  With rh_index_remap (rh particle j stands for lh
 * particle remap[j], as in neighborlist_changes) a pair whose lh particle is
 * itself remapped is kept only for i >= remap[j], and each edge (i, remap[j], s)
 * is written with its reverse (remap[j], i, -s) (_build_segmentation_mask
 * :505-539, _compact_edges :651-689); without it edges are (i, j), j indexing rh.
 * Rows past n_edges are padded with max(n_lh, n_rh); overflow is reported in
 * `status` (KUPS_CAP_EDGES, required = n_edges). */
size_t kups_neighborlist_rh_workspace_bytes(int64_t n_lh, int64_t n_rh, int32_t n_systems);
int32_t kups_neighborlist_build_rh(const double *lh_positions, const int32_t *lh_system,
                                   const int32_t *lh_inclusion, const int32_t *lh_exclusion, int64_t n_lh,
                                   const double *rh_positions, const int32_t *rh_system,
                                   const int32_t *rh_inclusion, const int32_t *rh_exclusion, int64_t n_rh,
                                   const int32_t *rh_index_remap, int32_t n_inclusion, const double *tril,
                                   const double *cutoffs, int32_t n_systems, int32_t *edges, int32_t *shifts,
                                   int64_t edge_capacity, int64_t *n_edges, void *workspace,
                                   size_t workspace_bytes, kups_status *status, void *stream);

/* kups_neighborlist_split_changes is the split step of neighborlist_changes
 * (src/kups/core/neighborlist.py:1425-1515) applied to the edges of the combined
 * rh call (lh = n original particles followed by the k proposed ones, rh = the
 * old copies of the changed particles p_idx followed by the proposed ones,
 * remap = [p_idx, n + arange(k)]): removed = edges with both ends < n; added =
 * edges with an end >= n and no end that is a changed particle's old copy;
 * indices n + m are rewritten to p_idx[m].  Both outputs are compacted in edge
 * order and padded with n; n_added / n_removed receive the counts (overflow of
 * a capacity is reported in `status`). */
size_t kups_neighborlist_split_workspace_bytes(int64_t edge_rows, int64_t n);
int32_t kups_neighborlist_split_changes(const int32_t *edges, const int32_t *shifts, const int64_t *n_edges,
                                        int64_t edge_rows, int64_t n, const int32_t *p_idx, int64_t k,
                                        int32_t *added_edges, int32_t *added_shifts, int64_t added_capacity,
                                        int64_t *n_added, int32_t *removed_edges, int32_t *removed_shifts,
                                        int64_t removed_capacity, int64_t *n_removed, void *workspace,
                                        size_t workspace_bytes, kups_status *status, void *stream);

/* ------------------------------------------------------------------------
 * Edge-set kernels of the local machine-learned potential (message passing
 * over the neighbour list; local_mliap_energy_full, src/kups/potential/mliap/
 * local.py:310-356).  Directed edges (i, j, s) as the neighbour list writes
 * them; rows past n_edges or with an index outside [0, n) are padding.
 *   kups_edge_vectors     d_e = x_j - x_i + s @ L (Edges.difference_vectors,
 *                         src/kups/core/neighborlist.py:164-184), float64 [E, 3]
 *                         (zero for padding rows)
 *   kups_edge_segment_sum out[i, :] = sum over edges with first index i of
 *                         values[e, :] (jax.ops.segment_sum), float64 [N, width],
 *                         written
 *   kups_edge_gradients   from g_e = dE/dd_e: dE/dx_j += g_e, dE/dx_i -= g_e and
 *                         dE/dL_ab += s_a g_b (Cartesian positions held fixed,
 *                         tril order), grad [N, 3] and grad_tril [S, 6] (may be
 *                         NULL) written
 * ------------------------------------------------------------------------ */
int32_t kups_edge_vectors(const double *positions, const int32_t *system, int64_t n, const double *tril,
                          int32_t n_systems, const int32_t *edges, const int32_t *shifts, int64_t n_edges,
                          double *d, void *stream);
int32_t kups_edge_segment_sum(const double *values, int32_t width, const int32_t *edges, int64_t n_edges,
                              int64_t n, double *out, void *stream);
int32_t kups_edge_gradients(const double *dE_dd, const int32_t *system, int64_t n, int32_t n_systems,
                            const int32_t *edges, const int32_t *shifts, int64_t n_edges, double *grad,
                            double *grad_tril, void *stream);

/* ------------------------------------------------------------------------
 * Lennard-Jones over an edge list — replaces lennard_jones_energy
 * (src/kups/potential/classical/lennard_jones.py:149-178) together with the
 * gradient PotentialFromEnergy obtains by jax.vjp with respect to
 * PositionAndUnitCell (src/kups/potential/common/energy.py:264-355).
 *
 *   species    i32 [n_particles]  index into the n_species x n_species tables
 *   sigma, epsilon f64 [n_species * n_species] (row-major, symmetric)
 *   energy     f64 [n_systems]        out: sum_edges E_e / 2
 *   grad       f64 [n_particles, 3]   out: dE/dx (zeroed by the call)
 *   grad_tril  f64 [n_systems, 6]     out: dE/dtril at fixed Cartesian x
 *   pair_fp32  non-zero: pair arithmetic in float32 (sums stay float64)
 * ------------------------------------------------------------------------ */
int32_t kups_lj_edges(const double *positions, const int32_t *system,
                      const int32_t *species, int64_t n_particles,
                      const double *tril, const double *cutoffs, int32_t n_systems,
                      const double *sigma, const double *epsilon, int32_t n_species,
                      const int32_t *edges, const int32_t *shifts, int64_t n_edges,
                      double *energy, double *grad, double *grad_tril,
                      int32_t pair_fp32, kups_status *status, void *stream);

/* ------------------------------------------------------------------------
 * Fused Lennard-Jones MD — replaces one or more calls of the propagator built
 * by make_velocity_verlet_step / make_baoab_langevin_step
 * (src/kups/md/integrators.py:273-318, 405-455) with the LJ potential and
 * neighbour list as derivative_computation
 * (src/kups/application/md/simulation.py:74-119).
 *
 * One persistent launch runs n_steps for every system.  Each CTA takes whole
 * systems from a work queue and keeps a system's atoms, periodic-image
 * copies and cell grid in shared memory for all its steps; the Verlet list
 * (cutoff + skin, uint16 indices) lives in the workspace, one region per
 * system, together with a per-system record (cell-sorted order, internal
 * positions, image copies, travelled distances) that lets the next call on
 * the same workspace resume without a list build (reuse_lists).  Pair
 * arithmetic is float32, per-system energy and virial sums float64.
 *
 * Atoms are stored sorted by system: system s owns [sys_offset[s],
 * sys_offset[s+1]).
 *   pos        float4 [n_atoms]  (x, y, z, species as int bits) in/out, Cartesian;
 *              returned wrapped into fractional [-0.5, 0.5) like
 *              MinimumImageConventionFlow (integrators.py:104-141)
 *   mom        float4 [n_atoms]  (px, py, pz, mass) in/out
 *   force      float4 [n_atoms]  (fx, fy, fz, -) in/out: F(t) on entry if
 *              forces_valid, else computed first; F(t + n dt) on exit
 *   sys_offset i32 [n_systems + 1]
 *   order      i32 [n_systems]   processing order (largest first balances load)
 *   tril       f32 [n_systems, 6]
 *   cutoff, skin, dt, kT, friction   f32 [n_systems]  (kT in eV, dt internal units)
 *   lj_table   f32 [n_species * n_species * 2]  (sigma^2, 4 epsilon)
 *   energy     f64 [n_systems]  out: potential energy at the last step
 *   kinetic    f64 [n_systems]  out: kinetic energy at the last step
 *   virial     f64 [n_systems, 6] out (may be NULL): dE/dtril at the last step
 *   trace_pe, trace_ke  f64 [n_steps, n_systems] out (may be NULL)
 *   rebuilds   i32 [n_systems] out (may be NULL): list builds during the call
 *   profile    u64 [10] out (may be NULL): clock64 cycles spent per phase (setup
 *              + first build, integrate, list/ghost update, forces, kick +
 *              reductions, write-back, and inside list builds: ghosts, binning,
 *              in-cell ordering, Verlet list), accumulated by each CTA's thread 0
 *   integrator 0 = velocity Verlet (NVE), 1 = BAOAB Langevin (NVT)
 *   seed, step0  counter-based (Philox4x32-10) noise: stream (seed, atom), counter step
 * ------------------------------------------------------------------------ */
typedef struct kups_md_args {
  void *pos;
  void *mom;
  void *force;
  const int32_t *sys_offset;
  const int32_t *order;
  const float *tril;
  const float *cutoff;
  const float *skin;
  const float *dt;
  const float *kT;
  const float *friction;
  const float *lj_table;
  double *energy;
  double *kinetic;
  double *virial;
  double *pressure;          /* [n_systems] out (may be NULL; needs virial): instantaneous
                                pressure 2K / 3V + Tr(stress) / 3 at the last step, stress =
                                -(sum_i dU/dr_i (x) r_i + h^T dU/dh) / V (md/observables.py:38-61,
                                observables/stress.py:70-82), energy / length^3 */
  double *trace_pe;
  double *trace_ke;
  int32_t *rebuilds;         /* [n_systems] out (may be NULL): Verlet-list builds per system */
  uint64_t *profile;         /* [10] out (may be NULL): SM cycles per phase, summed over CTAs */
  int64_t n_atoms;
  int32_t n_systems;
  int32_t n_species;
  int32_t n_steps;
  int32_t integrator;
  int32_t forces_valid;
  int32_t neighbor_capacity; /* Verlet-list slots per atom */
  uint64_t seed;
  uint64_t step0;
  int32_t n_ctas;            /* 0 = one per SM */
  int32_t block_threads;     /* 0 = library default */
  int32_t min_lanes_per_atom; /* lanes sharing one atom's Verlet list in the force phase:
                                 at least this many (1, 2, 4, 8 or 16; 0 = library default 2),
                                 more for small systems so every thread has work */
  int32_t reuse_lists;       /* 1: a system whose record in the workspace (written by the
                                previous call on the same workspace) matches this call's inputs
                                bit for bit (atom count, cell, cutoff, skin, lanes per atom,
                                neighbor_capacity, and every atom's wrapped position and
                                species) resumes with its cell-sorted order, image copies,
                                travelled distances and Verlet list instead of rebuilding them,
                                exactly as if the previous call had run on; 0: rebuild every
                                system.  Every call writes the records; integrator 3 always
                                rebuilds (the cell changes). */
  /* integrator 2 = CSVR (CSVRStep + velocity Verlet, md/integrators.py:469-640),
   * integrator 3 = CSVR + stochastic cell rescaling (make_csvr_npt_step, :641-890).
   * Per-system R1, R2 and the barostat's R are independent draws (the reference
   * draws one scalar per call for the whole batch). */
  const double *thermostat_tau;   /* [n_systems] tau_T (integrators 2, 3) */
  const double *target_pressure;  /* [n_systems] P0, energy / length^3 (integrator 3) */
  const double *barostat_tau;     /* [n_systems] tau_P (integrator 3) */
  const double *compressibility;  /* [n_systems] beta, length^3 / energy (integrator 3) */
  const double *min_scale;        /* [n_systems] mu clipped to [min_scale, 1 / min_scale] */
  double *cell;                   /* [n_systems, 6] in/out (integrator 3): float64 tril of the
                                     cell, scaled by the barostat; `tril` is not read */
  double *trace_virial;           /* [n_steps, n_systems, 6] out (may be NULL; integrators 0-2):
                                     dE/dtril after every step, as `virial` holds it after the
                                     last (the reference's potential returns it every step) */
  int64_t atom_base;              /* added to an atom's packed index where it keys the Langevin
                                     noise, and */
  int32_t system_base;            /* to the system index where it keys the thermostat and
                                     barostat draws: a call on systems [b, b + n_systems) of a
                                     larger batch (atoms from atom_base) draws the same numbers
                                     as the whole batch's call (0 for a whole batch) */
  int32_t pad_base;
} kups_md_args;

size_t kups_lj_md_workspace_bytes(const kups_md_args *args);
int32_t kups_lj_md_run(const kups_md_args *args, void *workspace, size_t workspace_bytes,
                       kups_status *status, void *stream);
/* Atoms of one system the fused kernel keeps in shared memory. */
int32_t kups_lj_md_max_atoms(void);

/* Layout conversion between the reference's particle table (float64 [N, 3]
 * positions / momenta / forces, float64 masses, int32 species; any order —
 * MDParticles, src/kups/application/md/data.py:31-65) and the packed float4
 * arrays of kups_lj_md_run.  perm[k] (may be NULL = identity) is the particle
 * index stored at packed slot k; force may be NULL (packed as zero / not
 * written back). */
int32_t kups_md_pack(const double *pos, const double *mom, const double *force,
                     const double *mass, const int32_t *species, const int32_t *perm,
                     int64_t n, void *pos4, void *mom4, void *force4, void *stream);
int32_t kups_md_unpack(const void *pos4, const void *mom4, const void *force4,
                       const int32_t *perm, int64_t n, double *pos, double *mom, double *force,
                       void *stream);

/* ------------------------------------------------------------------------
 * Ewald summation.
 *
 * kups_ewald_recip replaces ewald_long_range_energy with _structure_factor_full
 * (src/kups/potential/classical/ewald.py:394-439, 549-601), prefactor
 * (:363-391) and EwaldLongRangeInput.kvecs (:265-274), plus the jax.vjp
 * gradients with respect to positions and tril.  Atoms are grouped by system
 * (system s owns [sys_offset[s], sys_offset[s+1])).
 *   kvec_n     i32 [n_systems, n_kvecs, 3]  integer k coefficients (the
 *              reference's reciprocal_lattice_shifts; zero rows are padding)
 *   alpha      f64 [n_systems]; coulomb_k = HARTREE * BOHR (eV A / e^2)
 *   energy     f64 [n_systems] out;  grad f64 [N, 3] out (written, not added)
 *   grad_tril  f64 [n_systems, 6] out (may be NULL)
 *   structure_factor f64 [n_systems, n_kvecs, 2] out: S(k) (the EwaldCache
 *              structure_factor, float64 accumulation)
 * |n_a| <= 16 per axis.
 *
 * kups_ewald_self replaces ewald_self_interaction_energy (:277-302).
 *
 * kups_pair_edges evaluates, over a directed edge list, any sum of
 *   terms & 1: Lennard-Jones (lennard_jones.py:149-178),
 *   terms & 2: real-space Ewald K q_i q_j erfc(alpha r) / r (ewald.py:305-325),
 *   terms & 4: minus bare Coulomb K q_i q_j / r, the exclusion correction over
 *              intramolecular edges (ewald.py:328-346, coulomb.py:64-83),
 * each summed / 2 per system, with dE/dx (zeroed then accumulated) and
 * dE/dtril (may be NULL).  Distances and pair arithmetic in float64.
 * ------------------------------------------------------------------------ */
size_t kups_ewald_recip_workspace_bytes(int32_t n_systems, int32_t n_kvecs);
int32_t kups_ewald_recip(const double *positions, const double *charges,
                         const int32_t *sys_offset, int32_t n_systems,
                         int32_t max_atoms_per_system, const double *tril,
                         const int32_t *kvec_n, int32_t n_kvecs, const double *alpha,
                         double coulomb_k, double *energy, double *grad, double *grad_tril,
                         double *structure_factor, void *workspace, size_t workspace_bytes,
                         kups_status *status, void *stream);
/* kups_ewald_recip_energy: E = K sum_k P(k) |S(k)|^2 per system from given
 * structure factors (float64 [S, n_kvecs, 2]), the long-range energy of a
 * cached S(k) (EwaldCache / EwaldLongRangeComposer, src/kups/potential/
 * classical/ewald.py:86-150, 604-657); workspace as kups_ewald_recip. */
int32_t kups_ewald_recip_energy(const double *tril, const int32_t *kvec_n, int32_t n_kvecs, const double *alpha,
                                int32_t n_systems, double coulomb_k, const double *structure_factor,
                                double *energy, void *workspace, size_t workspace_bytes, kups_status *status,
                                void *stream);
/*
 * kups_ewald_recip_static — no counterpart in the reference.  The same
 * computation and outputs as kups_ewald_recip, for callers that cannot
 * allocate device memory and so cannot pass a workspace (e.g. an FFI handler
 * that receives only its input and output buffers).  Its scratch is one fixed
 * device array of KUPS_EWALD_RECIP_STATIC_SCRATCH_BYTES inside the library;
 * nothing is allocated or freed.
 *   - The scratch is 120 bytes of cell data per system (rounded up to 256
 *     bytes) plus 32 bytes per (system, k vector); sizes that need more than
 *     the array are refused with KUPS_ERR_CAPACITY before anything is
 *     launched (16 MiB holds, e.g., 512 systems x 1000 k vectors).
 *   - The first call on each device looks up the array's address with that
 *     device current; make that first call before any stream capture.  The
 *     address is kept per device for the life of the process: after a
 *     cudaDeviceReset the library must not be called on that device again.
 *   - The array is shared by all calls on a device and keeps the last call's
 *     contents; nothing in it needs to start at zero.  Calls that overlap in
 *     time (other streams or host threads) race on it: order them.
 *   - The array belongs to the library's Ewald module: every device on which
 *     any of this module's entry points runs (kups_ewald_recip, _static,
 *     _energy, kups_ewald_self, kups_pair_edges, kups_lj_ewald_real_forces*)
 *     holds its 16 MiB until the process exits.
 *   - Host-side returns, beyond the general KUPS_OK / KUPS_ERR_INVALID /
 *     KUPS_ERR_CUDA: KUPS_ERR_CAPACITY when the sizes need more than the
 *     array (nothing launched), KUPS_ERR_UNSUPPORTED for a device ordinal of
 *     64 or more.
 */
#define KUPS_EWALD_RECIP_STATIC_SCRATCH_BYTES ((size_t)16 << 20)
int32_t kups_ewald_recip_static(const double *positions, const double *charges,
                                const int32_t *sys_offset, int32_t n_systems,
                                int32_t max_atoms_per_system, const double *tril,
                                const int32_t *kvec_n, int32_t n_kvecs, const double *alpha,
                                double coulomb_k, double *energy, double *grad, double *grad_tril,
                                double *structure_factor, kups_status *status, void *stream);
int32_t kups_ewald_self(const double *charges, const int32_t *sys_offset, int32_t n_systems,
                        const double *alpha, double coulomb_k, double *energy, void *stream);
/* kups_lj_ewald_real_forces: the same real-space sum as kups_pair_edges with
 * terms 1 | 2 over the neighbour list at the cutoff, for systems grouped by
 * sys_offset whose cell widths are all at least twice the larger cutoff (every
 * pair within a cutoff is then its minimum image; otherwise the system is skipped
 * and KUPS_ERR_UNSUPPORTED is recorded): all pairs of a system in shared-memory
 * tiles, no stored list, float32 pair arithmetic (differences formed in
 * float64), energy [S] float64 (written), grad = dE/dx [N, 3] (written).
 * Used by the LJ + Ewald MD propagator; 1 <= n_species <= 8. */
int32_t kups_lj_ewald_real_forces(const double *positions, const double *charges, const int32_t *species,
                                  const int32_t *sys_offset, int32_t n_systems, int32_t max_atoms_per_system,
                                  const double *tril, const double *lj_sigma, const double *lj_epsilon,
                                  int32_t n_species, const double *lj_cutoff, const double *alpha,
                                  const double *ewald_cutoff, double coulomb_k, int32_t terms, double *energy,
                                  double *grad, kups_status *status, void *stream);
/* kups_lj_ewald_real_forces_packed: the same sum, arguments and outputs as
 * kups_lj_ewald_real_forces, with positions first stored in `workspace` as float
 * pairs hi = fl(x), lo = fl(x - hi) (differences (hj - hi) + (lj - li) keep float32
 * relative accuracy with no float64 arithmetic) and the pair terms evaluated only for
 * the partners a lane found inside the cutoff among 32 tested.  terms & 8 adds the
 * energy and gradient onto the caller's (e.g. the reciprocal-space result) instead
 * of writing them.  With terms & 8, bits 8-11 of terms give the number of partner
 * shares per block of 16 atoms (1-15: gridDim.z; the shares add their partial forces
 * with atomics, so the float summation order varies); 0 means one share.  Without
 * terms & 8 there is one share.  A system with more than
 * max_atoms_per_system atoms records KUPS_ERR_INVALID and is skipped.
 * Workspace: kups_lj_ewald_real_forces_workspace_bytes(n_systems, max_atoms). */
size_t kups_lj_ewald_real_forces_workspace_bytes(int32_t n_systems, int32_t max_atoms_per_system);
int32_t kups_lj_ewald_real_forces_packed(const double *positions, const double *charges,
                                         const int32_t *species, const int32_t *sys_offset,
                                         int32_t n_systems, int32_t max_atoms_per_system,
                                         const double *tril, const double *lj_sigma,
                                         const double *lj_epsilon, int32_t n_species,
                                         const double *lj_cutoff, const double *alpha,
                                         const double *ewald_cutoff, double coulomb_k, int32_t terms,
                                         double *energy, double *grad, void *workspace,
                                         size_t workspace_bytes, kups_status *status, void *stream);
/* kups_erfc_eval: out[i] = erfc(x[i]) for x >= 0 (float32) by the library's pair-term
 * erfc, the Chebyshev-fitted formula of Numerical Recipes in C (2nd ed., section 6.2),
 * fractional error below 1.2e-7 in exact arithmetic; exposed so its accuracy can be
 * checked against a float64 erfc. */
int32_t kups_erfc_eval(const float *x, int64_t n, float *out, void *stream);
int32_t kups_pair_edges(const double *positions, const int32_t *system, const int32_t *species,
                        const double *charges, int64_t n_particles, const double *tril,
                        int32_t n_systems, const double *lj_sigma, const double *lj_epsilon,
                        int32_t n_species, const double *lj_cutoff, const double *alpha,
                        const double *ewald_cutoff, double coulomb_k, int32_t terms,
                        const int32_t *edges, const int32_t *shifts, int64_t n_edges,
                        double *energy, double *grad, double *grad_tril, kups_status *status,
                        void *stream);

/* ------------------------------------------------------------------------
 * Bonded edge-set potentials — replace the energies of
 * src/kups/potential/classical/harmonic.py:83-163, morse.py:142-171,
 * cosine_angle.py:152-221, dihedral.py:214-273 and inversion.py:136-209 on the
 * HyperGraph of an EdgeSetGraphConstructor (potential/common/graph.py:289-361),
 * with the jax.vjp gradient of PotentialFromEnergy (common/energy.py:264-355).
 *   kind  order  params per species tuple (row-major table [T^order, params])
 *   0     2      harmonic bond   x0, k:             k (r - x0)^2
 *   1     2      Morse bond      r0, D, alpha:      D (1 - exp(-alpha (r - r0)))^2
 *   2     3      harmonic angle  theta0 [deg], k:   k (theta - theta0)^2, theta at atom 0
 *   3     3      cosine angle    theta0 [rad], K, linear_tol (UFF cosine form)
 *   4     4      dihedral        V, n, phi0:        V/2 (1 - cos(n phi0) cos(n phi))
 *   5     4      inversion       omega0, k          (UFF, atom 0 the centre)
 *   edges  i32 [n_edges, order]; shifts i32 [n_edges, order - 1, 3]: integer image
 *          shifts of atoms 1.. relative to atom 0 (Edges.shifts)
 *   energy f64 [n_systems], grad f64 [n_particles, 3], grad_tril f64 [n_systems, 6]
 *          (may be NULL): ADDED to (zero them first), so several terms can share
 *          one buffer; an edge belongs to the system of its atom 0.
 * Difference vectors and all sums in float64; the per-edge energy and gradient in
 * float64, or in float32 when fp32 != 0 (float32 relative error, about 1e-6 on the
 * energies; float64 is slow on this part).  An edge with an index or species out of
 * range records KUPS_ERR_INVALID (first offending edge) and is skipped. */
int32_t kups_bonded_order(int32_t kind);
int32_t kups_bonded_param_count(int32_t kind);
int32_t kups_bonded_edges(int32_t kind, const double *positions, const int32_t *system,
                          const int32_t *species, int64_t n_particles, const double *tril,
                          int32_t n_systems, const int32_t *edges, const int32_t *shifts,
                          int64_t n_edges, const double *params, int32_t n_species,
                          double *energy, double *grad, double *grad_tril, int32_t fp32,
                          kups_status *status, void *stream);

/* MC energy change of a bonded term for a patch of moved particles — replaces the
 * old-graph / new-graph pair of LocalGraphSumComposer over an EdgeSetGraphConstructor
 * with a probe (src/kups/potential/common/graph.py:336-361, 412-450).
 *   delta[s] += sum over edges with an atom in `changed` of E_e(new) - E_e(old), the
 *   edge's system being that of its atom 0 (zero delta first; terms add up).
 *   changed       i32 [n_changed] distinct particle indices (all systems in one call),
 *                 n_changed < 2^31 - 1
 *   new_positions f64 [n_changed, 3]
 *   new_image     i32 [n_changed, 3] or NULL: the lattice offset n with
 *                 new_position = unwrapped - n @ L when the move wrapped the atom; an
 *                 edge's shifts become s_m + n_{m+1} - n_0, as the reference's probe
 *                 rewrites the edge data
 *   incidence_offsets i64 [n_particles + 1], incidence_edges i32 [...] or both NULL:
 *                 the edges of particle i are incidence_edges[incidence_offsets[i] ..
 *                 incidence_offsets[i + 1]), each listed once; with them each changed
 *                 particle walks its own edges (an edge with several changed particles is
 *                 taken by the one earliest in `changed`), without them every edge is scanned
 * Positions are not modified.  Workspace: kups_bonded_delta_workspace_bytes(n_particles).
 * Other arguments as kups_bonded_edges; a changed index out of range records
 * KUPS_ERR_INVALID (first_bad = its position in `changed`). */
size_t kups_bonded_delta_workspace_bytes(int64_t n_particles);
int32_t kups_bonded_delta(int32_t kind, const double *positions, const int32_t *system,
                          const int32_t *species, int64_t n_particles, const double *tril,
                          int32_t n_systems, const int32_t *edges, const int32_t *shifts,
                          int64_t n_edges, const double *params, int32_t n_species,
                          const int64_t *incidence_offsets, const int32_t *incidence_edges,
                          const int32_t *changed, const double *new_positions,
                          const int32_t *new_image, int64_t n_changed, double *delta, int32_t fp32,
                          void *workspace, size_t workspace_bytes, kups_status *status,
                          void *stream);

/* ------------------------------------------------------------------------
 * Integrator building blocks on the float64 particle table (systems larger
 * than kups_lj_md_max_atoms, Ewald MD): MomentumStep (p -= dE/dx * dt * scale),
 * PositionStep + MinimumImageConventionFlow (r += p/m * dt * scale, wrapped
 * into fractional [-0.5, 0.5)) and StochasticStep (Ornstein-Uhlenbeck)
 * (src/kups/md/integrators.py:104-401).  dt, kT, friction are per system.
 * ------------------------------------------------------------------------ */
int32_t kups_md_kick(double *momenta, const double *grad, const int32_t *system,
                     const double *dt, double scale, int64_t n_particles, void *stream);
int32_t kups_md_drift(double *positions, const double *momenta, const double *masses,
                      const int32_t *system, const double *dt, const double *tril, double scale,
                      int64_t n_particles, void *stream);
int32_t kups_md_thermostat(double *momenta, const double *masses, const int32_t *system,
                           const double *dt, const double *kT, const double *friction,
                           uint64_t seed, uint64_t step, int64_t n_particles, void *stream);
/* kups_md_thermostat with the step (the noise counter) read from device memory when the
 * kernel runs: a captured CUDA graph that also advances *step replays successive steps. */
int32_t kups_md_thermostat_counted(double *momenta, const double *masses, const int32_t *system,
                                   const double *dt, const double *kT, const double *friction,
                                   uint64_t seed, const uint64_t *step, int64_t n_particles, void *stream);

/* ------------------------------------------------------------------------
 * Virial observables per system — replaces stress_via_virial_theorem,
 * molecular_stress_via_virial_theorem and stress_via_lattice_vector_gradients
 * (src/kups/observables/stress.py:64-118, 139-190), particle_kinetic_energy summed
 * per system and instantaneous_pressure (src/kups/md/observables.py:17-61).
 *
 *   stress            sigma_ab = -(sum_i r_ia g_ib + (L^T G)_ab) / V
 *   molecular_stress  -(sym(sum_i w_i (x) g_i) + L^T G) / V, sym(A) = (A + A^T) / 2,
 *                     w_i = r_i - wrap(r_i - R_g), R_g the wrapped centre of the
 *                     atom's group (RASPA convention)
 *   lattice_stress    -G / V
 *   kinetic           sum_i |p_i|^2 / (2 m_i)
 *   pressure          2 K / (3 V) + Tr(stress) / 3 (K = 0 when momenta is NULL)
 * g = dU/dx f64 [n_particles, 3], G = dU/dL from grad_tril f64 [n_systems, 6]
 * (NULL: zero), V = |L00 L11 L22| of each system (the reference divides the
 * molecular stress of every system by the first system's volume, stress.py:114).
 * Outputs f64 [n_systems, 9] (row-major 3x3) or [n_systems]; each may be NULL.
 * group i32 [n_particles] in [0, n_groups) is read only for molecular_stress;
 * momenta f64 [n_particles, 3] and masses f64 [n_particles] may be NULL unless
 * kinetic is asked for.  A particle with a system or group out of range records
 * KUPS_ERR_INVALID and is skipped.  Workspace:
 * kups_virial_stress_workspace_bytes(n_systems, molecular_stress ? n_groups : 0).
 * ------------------------------------------------------------------------ */
size_t kups_virial_stress_workspace_bytes(int32_t n_systems, int32_t n_groups);
int32_t kups_virial_stress(const double *positions, const double *grad, const int32_t *system,
                           int64_t n_particles, const double *tril, const double *grad_tril,
                           int32_t n_systems, const int32_t *group, int32_t n_groups,
                           const double *momenta, const double *masses, double *stress,
                           double *molecular_stress, double *lattice_stress, double *kinetic,
                           double *pressure, void *workspace, size_t workspace_bytes,
                           kups_status *status, void *stream);

/* ------------------------------------------------------------------------
 * Batched grand-canonical Monte Carlo of one rigid molecule species in rigid
 * frameworks (LJ + Ewald + LJ tail correction, muVT ensemble) — replaces
 * MCMCPropagator.__call__ with the moves of make_gcmc_mcmc_propagator
 * (src/kups/core/propagator.py:312-345, src/kups/mcmc/moves.py:1078-1230),
 * the incremental potential (src/kups/potential/common/graph.py:419-453,
 * src/kups/potential/classical/ewald.py:442-486), MuVTLogProbabilityRatio
 * (src/kups/mcmc/probability.py:176-225) and acceptance_target_schedule
 * (src/kups/core/parameter_scheduler.py:161-208).  One launch runs n_steps
 * MC steps of every system (one CTA per system).
 *
 * Guests of system s occupy slots [0, n_mol[s]) of guest_pos
 * [n_systems, max_mol, atoms_per_mol] (float4 x, y, z, species bits); a
 * deletion moves the last molecule into the freed slot.  Framework atoms of
 * system s are fw_pos[fw_start[s] .. + fw_count[s]] (systems may share them).
 * Move kinds: 0 translate, 1 rotate, 2 reinsert, 3 insert, 4 delete;
 * move_cum = cumulative probabilities of translate, rotate, reinsert
 * (the rest is exchange, split evenly between insert and delete).
 * Schedulers 0..3 = translate, rotate, reinsert, exchange: width[s*4+k],
 * width_max[s*4+k] (<= 0: unbounded), history (bits) [s*4+k][4 words],
 * history_index [s*4+k].
 * With `proposals` non-NULL (one per system) the moves are taken from there
 * instead of the generator (tests / replays); out_delta[s] = (dE, dE_real,
 * dE_recip, log acceptance) of the last step.
 * ------------------------------------------------------------------------ */
typedef struct kups_gcmc_proposal {
  int32_t kind;
  int32_t mol;
  int32_t force_reject;
  int32_t pad;
  float pos[8][4]; /* new positions (x, y, z, species bits) of the molecule */
} kups_gcmc_proposal;

/* One record per (step, system) written when kups_gcmc_args.trace is set,
 * at trace[step * n_systems + s]: what the step proposed and decided, so a
 * replay can check the move generator, ln acc and the accept decision. */
typedef struct kups_gcmc_trace {
  int32_t kind;      /* 0 translate, 1 rotate, 2 reinsert, 3 insert, 4 delete */
  int32_t mol;       /* molecule slot moved, inserted into or deleted (-1: none) */
  int32_t accept;
  int32_t n_mol;     /* molecules before the step */
  int32_t has_old;   /* the move removes an existing molecule's old position */
  int32_t has_new;   /* the move places a molecule (new_pos valid) */
  float width;       /* step width of the move's scheduler when proposed */
  int32_t pad;
  double de;         /* energy change of the proposal */
  double log_p;      /* ln acc (muVT + proposal ratio) */
  double log_u;      /* ln u of the uniform in (0, 1] it was compared with */
  double ln_ratio;   /* log proposal ratio of the learned density (0: uniform) */
  float new_pos[8][4];
} kups_gcmc_trace;

typedef struct kups_gcmc_args {
  const void *fw_pos;           /* float4 */
  const float *fw_charge;
  const int32_t *fw_start;
  const int32_t *fw_count;
  void *guest_pos;              /* float4 [S, max_mol, apm] in/out */
  int32_t *n_mol;               /* [S] in/out */
  const void *motif_pos;        /* float4 [apm]: template (x, y, z, species bits) */
  const float *motif_charge;    /* [apm] */
  const double *motif_species_count; /* [n_species] */
  const double *fw_species_count;    /* [S, n_species] */
  const double *tril;           /* [S, 6] */
  const double *rc_lj;          /* [S] */
  const double *rc_ew;          /* [S] */
  const double *alpha;          /* [S] */
  const int32_t *kvec_n;        /* [S, n_kvecs, 3] */
  const double *prefactor;      /* [S, n_kvecs] P(k) */
  double *structure_factor;     /* [S, n_kvecs, 2] in/out */
  const float *lj_table;        /* [n_species^2 * 2]: sigma^2, 4 eps */
  const double *tail_coef;      /* [S, n_species^2] or NULL */
  const double *self_energy_mol;      /* [S] self energy of one molecule */
  const double *exclusion_energy_mol; /* [S] intramolecular exclusion correction */
  const double *kT;             /* [S] */
  const double *log_activity;   /* [S] ln(f / kT) */
  double *energy;               /* [S] in/out */
  float *width;                 /* [S, 4] */
  const float *width_max;       /* [S, 4] */
  uint32_t *history;            /* [S, 4, 4] */
  int32_t *history_index;       /* [S, 4] */
  int64_t *attempted;           /* [S, 5] */
  int64_t *accepted;            /* [S, 5] */
  const kups_gcmc_proposal *proposals; /* [S] or NULL */
  double *out_delta;            /* [S, 4] or NULL */
  const float *proposal_node;   /* [G^3] learned insertion density (kups_mlp_grid_norm) or NULL */
  const double *proposal_cdf;   /* [G^3 + 1] */
  void *workspace;              /* float2 [3, S, n_kvecs] scratch (a reserved slab, then float32
                                   mirrors of S(k) and of P(k) with the packed k vector) */
  const void *fw_group;         /* float4 [host atoms / 32][2] or NULL: per 32 host atoms
                                   (blocks start on multiples of 32) the fractional centre and
                                   per-axis half extents; used when every cell width is at
                                   least twice the cutoffs, to skip groups beyond the cutoff */
  double *obs_sums;             /* [S, 5] in/out or NULL: after every step adds U, N, U N, N^2
                                   and U^2 (U = energy[s], N = n_mol[s]): the block sums behind
                                   the reference's per-step energy / loading / heat-of-adsorption
                                   analysis (application/mcmc/analysis.py:82-158) */
  float move_cum[3];
  float pad0;
  double coulomb_k;
  uint64_t seed;
  uint64_t step0;
  int32_t n_systems;
  int32_t max_mol;
  int32_t atoms_per_mol;
  int32_t n_species;
  int32_t n_kvecs;
  int32_t n_steps;
  int32_t history_len;
  int32_t proposal_grid;        /* G; with proposal_node set, insertions draw the molecule's
                                   centre (atom mean) from the grid density q and add
                                   -ln(V q) to ln acc, deletions add +ln(V q) */
  kups_gcmc_trace *trace;       /* [n_steps, S] or NULL: per-step record of every system */
  int32_t block_threads;        /* threads per system's CTA: 64, 128 or 256 (0: 128); the
                                   launch-shape autotuner picks one per workload */
  int32_t pad1;
  unsigned long long *profile;  /* [6] or NULL: clock cycles of thread 0 summed over all systems
                                   and steps per phase (proposal, host atoms, guests and the
                                   moved molecule, phase tables, k sum, acceptance and commit) */
  double *host_cache;           /* [S, max_mol, 2] in/out or NULL: per guest molecule its real-space
                                   energy with the (rigid) host and a 64-bit key of the atom
                                   positions it belongs to (bits in the second double; zeros =
                                   no entry).  With every cell width at least twice the cutoffs,
                                   a move reads the old molecule's host energy from its entry
                                   when the key matches the molecule's positions, and computes
                                   only the new positions against the host; entries follow
                                   their molecules (written on acceptance, moved on deletion,
                                   filled on a miss).  A hit equals the recomputed value bit for
                                   bit; stale or foreign entries only miss.  NULL: both ends
                                   are computed every move */
  int32_t k_shared;             /* 1: every system has the same k vectors and P(k) (replicas of
                                   one cell): the float32 (P(k), packed k) mirror in the workspace
                                   is kept once, in system 0's slot, and read by every system */
  int32_t pad2;
} kups_gcmc_args;

int32_t kups_gcmc_run(const kups_gcmc_args *args, kups_status *status, void *stream);

/* kups_lj_tail_correction replaces global_lennard_jones_tail_correction_energy
 * and _pressure (potential/classical/lennard_jones.py:276-340): per system
 * (atoms grouped by sys_offset) the analytic long-range energy and pressure of
 * the species pairs with tail_mask[a * T + b] != 0 (NULL: pairs with eps > 0),
 * float64; energy / pressure [S] (either may be NULL).  1 <= n_species <= 64. */
int32_t kups_lj_tail_correction(const int32_t *species, const int32_t *sys_offset, int32_t n_systems,
                                const double *tril, const double *sigma, const double *epsilon,
                                const int32_t *tail_mask, int32_t n_species, const double *cutoff,
                                double *energy, double *pressure, kups_status *status, void *stream);

/* ------------------------------------------------------------------------
 * Tensor-core GEMM (tcgen05, BF16 inputs, FP32 accumulation in tensor memory)
 * used by the learned insertion proposal (no counterpart in the reference;
 * the proposal enters through the ChangesFn log-ratio of the insertion move,
 * src/kups/mcmc/moves.py:92-98 and src/kups/core/propagator.py:330-334).
 *   C[m, n] = act(alpha * sum_k A[m, k] B[n, k] + beta * C[m, n] + bias[n]) * gate'
 * Operands are addressed element-wise as p[r * s_row + c * s_col] (any
 * transposition); *_bf16 selects bfloat16 (else float32) storage.
 * act: 0 none, 1 ReLU, 2 softplus.  gate_kind 1 / 2 multiplies by the ReLU /
 * softplus derivative of gate[m, n] (backward passes); 3 by the softplus
 * derivative written through the layer's output h = gate[m, n]: 1 - exp(-h).
 * c2 (may be NULL) is a second copy of C with its own strides and type.
 * split_k > 1 splits K over CTAs that atomically add alpha * partial into a
 * float32 C (beta must be 1, no act / bias / gate / c2); zero C first to get
 * the plain product.
 * Bfloat16 operands with K contiguous (16-byte aligned, row strides multiples of
 * 8 elements) and a row-major float32 C with N a multiple of 32 (and beta = 0
 * unless split) are loaded by TMA into 128-byte swizzled tiles; every other
 * layout is staged element-wise.  Results agree to the float32 accumulation
 * order either way.
 * ------------------------------------------------------------------------ */
int32_t kups_gemm_bf16(const void *a, int32_t a_bf16, int64_t sa_row, int64_t sa_col,
                       const void *b, int32_t b_bf16, int64_t sb_row, int64_t sb_col,
                       void *c, int32_t c_bf16, int64_t sc_row, int64_t sc_col, void *c2,
                       int32_t c2_bf16, int64_t sc2_row, int64_t sc2_col, const float *bias,
                       const float *gate, int32_t gate_kind, int64_t sg_row, int64_t sg_col,
                       int32_t m, int32_t n, int32_t k, float alpha, float beta, int32_t act,
                       int32_t split_k, kups_status *status, void *stream);

/* ------------------------------------------------------------------------
 * Learned insertion proposal (no counterpart in the reference; its density
 * enters the exchange move's log proposal ratio, the ChangesFn hook of
 * src/kups/mcmc/moves.py:92-98 summed at src/kups/core/propagator.py:330-334).
 *
 * Network (fixed): 64 Fourier features (sin, cos)(2 pi m_j . f) of the
 * fractional position f for 32 integer vectors freq[j] = m_j, three softplus
 * layers of width 256 on the tensor cores (bfloat16 operands, float32
 * accumulation), linear output g(f).  Flat float32 parameters, offsets:
 *   W1 [256, 64] at 0, b1 at 16384, W2 [256, 256] at 16640, b2 at 82176,
 *   W3 [256, 256] at 82432, b3 at 147968, w4 [256] at 148224, b4 at 148480.
 * Training minimises the noise-contrastive loss over equal halves of data
 * and uniform points, L = mean softplus(-g) (data) + mean softplus(g)
 * (uniform), whose minimiser is g = ln p_data on the unit cube.
 * ------------------------------------------------------------------------ */
#define KUPS_MLP_PARAMS 148481
typedef struct kups_mlp {
  float *param;        /* [KUPS_MLP_PARAMS] float32 master copy */
  void *param_bf16;    /* [KUPS_MLP_PARAMS] bfloat16 copy the GEMMs read */
  float *grad;         /* [KUPS_MLP_PARAMS] accumulated by kups_mlp_bwd, zeroed by kups_mlp_adam */
  float *adam_m;       /* [KUPS_MLP_PARAMS] */
  float *adam_v;       /* [KUPS_MLP_PARAMS] */
  const int32_t *freq; /* [32, 3] integer frequency vectors */
  void *param_bf16_t;  /* [2, 256, 256] bfloat16 W2^T, W3^T (kept by init / Adam) */
} kups_mlp;

/* workspace for kups_mlp_fwd / kups_mlp_bwd / kups_mlp_grid_norm over n points
 * (forward passes run in chunks of at most 65536 points) */
size_t kups_mlp_workspace_bytes(int64_t n_points);
/* weights uniform with variance 1 / fan_in from Philox(seed), biases, moments, gradient zero */
int32_t kups_mlp_init(const kups_mlp *net, uint64_t seed, void *stream);
/* g [n] (float32) at fractional points x [n, 3] (float64) */
int32_t kups_mlp_fwd(const kups_mlp *net, const double *x, int64_t n, float *g, void *workspace,
                     size_t workspace_bytes, kups_status *status, void *stream);
/* training batch: rows [0, batch/2) drawn with replacement from data [n_data, 3]
 * (label 1), rows [batch/2, batch) uniform in [0, 1)^3 (label 0); batch even */
int32_t kups_mlp_nce_batch(const double *data, int64_t n_data, int32_t batch, uint64_t seed,
                           uint64_t step, double *x, float *label, void *stream);
/* forward + backward of the loss over n <= 65536 labelled points: adds dL/dparam
 * to net->grad and L to *loss (loss may be NULL) */
int32_t kups_mlp_bwd(const kups_mlp *net, const double *x, const float *label, int32_t n, float *loss,
                     void *workspace, size_t workspace_bytes, kups_status *status, void *stream);
/* Adam step t >= 1 (Kingma & Ba); refreshes param_bf16 and zeroes grad */
int32_t kups_mlp_adam(const kups_mlp *net, int64_t t, float lr, float beta1, float beta2, float eps,
                      void *stream);
/* Grid density for the sampler: node[(i G + j) G + k] = exp(temper (g(i/G, j/G, k/G) - max g))
 * + floor_frac * mean (so every cell has positive mass), cdf [G^3 + 1] = running
 * sums of cell masses (mean of the 8 corners), float64.  2 <= G <= 256; temper > 0
 * flattens (< 1) or sharpens (> 1) the learned density. */
int32_t kups_mlp_grid_norm(const kups_mlp *net, int32_t grid, float temper, float floor_frac,
                           float *node, double *cdf, void *workspace, size_t workspace_bytes,
                           kups_status *status, void *stream);
/* n exact draws f [n, 3] from the piecewise-trilinear grid density (cell by its
 * mass, corner by its value, per-axis sqrt transform) with ln q_f(f), the
 * density in fractional measure (the insertion's log ratio is -ln q_f) */
int32_t kups_proposal_sample(const float *node, const double *cdf, int32_t grid, int64_t n,
                             uint64_t seed, double *f, double *log_q, void *stream);
/* ln q_f at fractional points f [n, 3] (any periodic image) */
int32_t kups_proposal_log_density(const float *node, const double *cdf, int32_t grid, const double *f,
                                  int64_t n, double *log_q, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* KUPS_GB300_H */
