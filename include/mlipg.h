/*
 * mlipg: linearized-MLIP ("gtinv") energy / force / virial evaluation on one
 * NVIDIA GB300 (sm_103a), as a plain C ABI.
 *
 * Drop-in for the LAMMPS path `pair_style mlip_gtinv` +
 * `pair_coeff * * <mlp.lammps> El1 ... ElN` of the reference package
 * (quantum-mtl/lammps-mlip-package).  Every entry point below names the
 * reference interface it replaces (file:line in that package).
 *
 * Conventions
 *  - Every function returns an int status (MLIPG_OK = 0); on failure the
 *    message is available from mlipg_last_error().  Nothing calls exit().
 *  - Host arrays are owned by the caller; the library owns grow-only device
 *    buffers and one CUDA stream per handle.  A handle is not re-entrant:
 *    use one handle per thread / MPI rank.
 *  - Positions are in Angstrom, energies in eV, forces in eV/Angstrom;
 *    the virial is -sum r_ij (x) f_ij in LAMMPS order xx yy zz xy xz yz.
 */
#ifndef MLIPG_H_
#define MLIPG_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mlipg_handle mlipg_handle;

enum mlipg_status {
  MLIPG_OK = 0,
  MLIPG_EINVAL = 1,    /* bad argument */
  MLIPG_EIO = 2,       /* potential file unreadable or malformed */
  MLIPG_ENOMEM = 3,    /* device or pinned host allocation failed */
  MLIPG_ECUDA = 4,     /* CUDA runtime error */
  MLIPG_ENOTSUP = 5,   /* model outside what the kernels support */
  MLIPG_ECAPACITY = 6, /* neighbour count above the kernel's capacity */
  MLIPG_ENOGPU = 7,    /* no usable CUDA device */
  MLIPG_ETIMEDOUT = 8, /* a wait ran past its deadline */
  MLIPG_EBUSY = 9      /* request queue full / budget exhausted */
};

enum mlipg_precision {
  MLIPG_PREC_FP64 = 0,      /* FP64 results: radial functions, Y_lm, order
                               parameters, the polynomial, forces, energies
                               and virial in FP64; the invariant and adjoint
                               products in double-float arithmetic (FP32
                               pairs, 48-bit significands, a few 2^-47
                               relative error per operation, on the FP32
                               pipe) with the adjoint summed in exact fixed
                               point (order independent).  Agrees with the
                               all-FP64 form to ~1e-13 relative. */
  MLIPG_PREC_MIXED = 1,     /* FP32 radial/Y_lm/invariant/adjoint products;
                               order-parameter neighbour sums (Kahan) and unit
                               energies (TwoSum) in compensated FP32, at FP32
                               pipe speed; the polynomial's input features
                               and their energy in FP64 (FP64 order
                               parameters); force, per-atom and total energy
                               and virial accumulation in FP64.  Energy error:
                               a few FP32 ulps of sum |w_f| |d_f| over the
                               other (linear-only) features */
  MLIPG_PREC_MIXED_A64 = 2, /* as MLIPG_PREC_MIXED, with the order-parameter
                               neighbour sums made with plain FP64 FMAs */
  MLIPG_PREC_FP64_NATIVE = 3 /* every product and sum in native FP64 (the
                               reference's arithmetic, at the FP64 pipe's
                               rate: 1/64 of FP32 on GB300) */
};

/* Message of the last failure on this handle (h may be NULL for failures
 * of mlipg_create or of calls without a handle; thread-local). */
const char* mlipg_last_error(const mlipg_handle* h);

/* Reads a potential file (mlp.lammps format) and uploads the model.
 * Replaces read_potential_file + MLIPModel::initialize
 * (src/USER-MLIP/mlipkk_potential_parser.cpp:14-105, mlipkk.cpp:27-53,
 *  called from PairMLIPGtinvKokkos::coeff, pair_mlip_gtinv_kokkos_impl.h:92-144). */
int mlipg_create(const char* potential_path, int precision, mlipg_handle** out);

/* Releases device memory and the stream.  (~PairMLIPGtinvKokkos,
 * pair_mlip_gtinv_kokkos_impl.h:60-85) */
int mlipg_destroy(mlipg_handle* h);

/* Switches between the precisions of enum mlipg_precision. */
int mlipg_set_precision(mlipg_handle* h, int precision);

/* Elements of the potential file, their masses and the cutoff radius.
 * (element list / masses: mlipkk_potential_parser.cpp:26-39,100-102;
 *  cutoff for init_one: pair_mlip_gtinv_kokkos_impl.h:214-221) */
int mlipg_num_elements(const mlipg_handle* h);
const char* mlipg_element_name(const mlipg_handle* h, int k);
double mlipg_element_mass(const mlipg_handle* h, int k);
double mlipg_cutoff(const mlipg_handle* h);

/* Maps LAMMPS atom types 1..n_lmp_types to file elements by name, exactly
 * like the trailing arguments of `pair_coeff * * file El1 ... ElN`;
 * "NULL" leaves a type unhandled.  Unknown names are an error ("No matching
 * element in Machine Learning Interatomic Potential file"); all-NULL is an
 * error ("Incorrect args for pair coefficients").
 * (pair_mlip_gtinv_kokkos_impl.h:146-195) */
int mlipg_set_type_map(mlipg_handle* h, int n_lmp_types, const char* const* element_names);

/* One force evaluation on LAMMPS host arrays ("neigh full newton on").
 *   x[nall*3], type[nall] (1-based LAMMPS types), full neighbour list
 *   inum/ilist/numneigh/firstneigh (entries masked with NEIGHMASK).
 * Outputs: f[nall*3] is ACCUMULATED (ghost forces included, to be reverse-
 * communicated as LAMMPS does); *energy and virial[6] are overwritten when
 * eflag / vflag are non-zero; eatom[nlocal] and vatom[nlocal][6] (LAMMPS order)
 * are accumulated if not NULL.  Per-atom virials attribute each pair's
 * -r_ij (x) f_ij to the atom whose adjoint produced f_ij (the reference
 * allocates but never fills eatom/vatom, pair_mlip_gtinv_kokkos_impl.h:287-296).
 * Replaces PairMLIPGtinvKokkos::compute (pair_mlip_gtinv_kokkos_impl.h:272-406)
 * with set_structure (:411-599), MLIPModelLMP::compute (mlipkk_lmp.h:145-228),
 * get_forces (:601-634) and get_stress (mlipkk_lmp.h:942-955). */
int mlipg_compute(mlipg_handle* h, int nlocal, int nall, const double* x, const int* type,
                  int inum, const int* ilist, const int* numneigh, const int* const* firstneigh,
                  int eflag, int vflag, double* f, double* energy, double* virial,
                  double* eatom, double* vatom);

/* Same evaluation on device-resident data, stream-ordered on the handle's
 * stream (no host synchronisation; capturable in a CUDA graph).
 *   d_x4[nall]: x, y, z and the element index as a double (< 0: skip);
 *   d_centers[ncenters]; CSR d_nbr_off[ncenters+1], d_nbr_idx[...];
 *   d_img (optional, NULL): packed periodic image per pair,
 *     code = (n1+512) | (n2+512)<<10 | (n3+512)<<20, 0 = no shift, applied
 *     with the lattice rows d_cell[9*d_center_cell[c]] of the centre's cell;
 *   d_fold (optional, NULL): atom -> force row (ghost -> owner).
 *   d_f[nforce*3] accumulated; d_eatom[ncenters] and d_vatom[ncenters][6]
 *   (LAMMPS order) written (optional);
 *   d_out8: [energy, virial xx yy zz yz zx xy, status] written; d_out8[7]
 *     holds the launch's status bits as a double (0 = clean; 1: an atom had
 *     more neighbours inside the cutoff than nb_cap, its energy and forces
 *     were skipped; 2: an element index outside the potential's elements;
 *     4: mixed or double-float path, adjoint outside the fixed-point
 *     range).  The call only enqueues work: read d_out8[7] after
 *     synchronising the stream, or call mlipg_device_status.
 * No counterpart in the reference (its device stages are internal,
 * mlipkk_lmp.h:145-228); this is the entry used by MD loops and batching. */
int mlipg_compute_device(mlipg_handle* h, int ncenters, const void* d_x4, const int* d_centers,
                         const int* d_nbr_off, const int* d_nbr_idx, const int* d_img,
                         const double* d_cell, const int* d_center_cell, const int* d_fold,
                         int nb_cap, double* d_f, double* d_eatom, double* d_vatom,
                         double* d_out8);

/* Allocation-free variant of mlipg_compute_device, for callers that cannot
 * let the library call cudaMalloc (device memory owned by the caller's own
 * pool or budget; latency-critical loops that must not enter the CUDA
 * allocator).  Same arguments and outputs as mlipg_compute_device; the
 * kernel's scratch (per-CTA partial sums and the status word) is a
 * file-scope device array of 2048 CTA slots (128 KiB) that every GPU
 * loading the library keeps until exit.  Launches needing more CTA slots
 * fail with MLIPG_ECAPACITY.  All calls share that array: calls that overlap
 * on the GPU race.  The first call on a device resolves the array's device
 * address (cudaGetSymbolAddress); make it before any stream capture.  The
 * calling thread's current device must be the handle's (MLIPG_EINVAL
 * otherwise); the resolved address is kept per device and is stale after a
 * cudaDeviceReset.  d_out8[7] carries the status bits as for
 * mlipg_compute_device.
 * No counterpart in the reference. */
int mlipg_compute_device_noalloc(mlipg_handle* h, int ncenters, const void* d_x4,
                                 const int* d_centers, const int* d_nbr_off,
                                 const int* d_nbr_idx, const int* d_img, const double* d_cell,
                                 const int* d_center_cell, const int* d_fold, int nb_cap,
                                 double* d_f, double* d_eatom, double* d_vatom, double* d_out8);

/* The handle's CUDA stream (cudaStream_t) for ordering caller work. */
void* mlipg_stream(mlipg_handle* h);

/* Status bits of the handle's last fused-kernel launch (any entry point):
 * waits for the handle's stream, then reads the launch's status word
 * (1 neighbour capacity, 2 element index, 4 fixed-point adjoint range; the
 * same value as that launch's d_out8[7]).  MD runs, batches and served
 * requests check the word themselves and fail with MLIPG_ECAPACITY,
 * MLIPG_EINVAL or MLIPG_ENOTSUP. */
int mlipg_device_status(mlipg_handle* h, int* bits);

/* Number of regression coefficients / structural features implied by a
 * model specification (MLIPPolynomial::get_n_coeffs,
 * mlipkk_potential_parser.cpp:107-116).  No GPU needed. */
int mlipg_count_coefficients(int n_types, int model_type, int maxp, int maxl, int gtinv_order,
                             const int* gtinv_maxl, const int* gtinv_sym, int n_fn,
                             long long* n_coeffs, long long* n_features);

/* Model sizes: out[0..12] = T, F, L, Lh, n_irreps, n_terms, n_folded_terms,
 * n_itc, D, n_coeffs, model_type, maxp, max_nonlinear_itc. */
int mlipg_model_info(const mlipg_handle* h, long long* out13);

/* Flattened model structure for cross-checks: irreps x typecomb list
 * [irreps, q, tc_0..tc_{q-1}]... and polynomial index [order, f...]...;
 * returns the number of ints (out may be NULL to query). */
long mlipg_dump_itc(const mlipg_handle* h, int* out, long cap);
long mlipg_dump_poly(const mlipg_handle* h, int* out, long cap);

/* Algorithmic FLOPs per atom step for element `elem` with nbar neighbours
 * (invariants and adjoint counted on the raw coupling table), and the same
 * count on the folded table the kernels execute (each conjugate pair of
 * terms once).  Measurement support; no reference counterpart. */
double mlipg_flops_per_atom_step(const mlipg_handle* h, int elem, double nbar);
double mlipg_flops_per_atom_step_executed(const mlipg_handle* h, int elem, double nbar);

/* Per-launch device time of the fused kernel: when on, every launch is
 * bracketed by CUDA events on the handle's stream; mlipg_kernel_times copies
 * the durations (ms) of the launches since the last call and clears them.
 * Returns the number copied.  Measurement support; no reference counterpart. */
int mlipg_set_profiling(mlipg_handle* h, int on);
int mlipg_kernel_times(mlipg_handle* h, float* ms, int cap);
/* With profiling on, SM cycles (summed over CTAs, thread-0 view) the fused
 * kernel spent in its phases since the last call: [0] neighbour compaction,
 * [1] order parameters, [2] nonlinear features + polynomial, [3] invariants
 * and adjoint of the tuple-batched units (warp 0's share), [4] the remaining
 * single-tuple units and the wait for the other warps, [5] forces and
 * reductions. */
int mlipg_phase_cycles(mlipg_handle* h, unsigned long long* out8);

/* Live FMA throughput of the CUDA-core FP32 (fp64 = 0) or FP64 (fp64 = 1)
 * pipe on the current device, in TFLOP/s: the roofline denominator of the
 * fused kernel.  Measurement support; no reference counterpart. */
int mlipg_measure_fma_peak(int fp64, double* tflops);

/* Many independent periodic cells (uneven atom counts) evaluated in one
 * persistent launch.  mlipg_batch_create wraps each cell's atoms into its cell
 * (lattices: 9 doubles per cell, rows a1 a2 a3), builds image-coded full
 * lists (no ghost atoms; small cells see their own images) and uploads
 * everything once.  mlipg_batch_compute evaluates all cells: energies[ncells]
 * (eV), forces[natoms_total*3] (eV/A) and virials[ncells*6] (LAMMPS order)
 * back on the host; mlipg_batch_launch only enqueues the evaluation on the
 * handle's stream and mlipg_batch_results copies the results of the last
 * launch (waiting for it); mlipg_batch_device_bytes is its device footprint.  No counterpart in the reference (one structure per
 * MLIPModel::set_structure call, mlipkk.cpp:278-372). */
typedef struct mlipg_batch mlipg_batch;
int mlipg_batch_create(mlipg_handle* h, int ncells, const int* natoms, const double* lattices,
                       const double* x, const int* elements, mlipg_batch** out);
int mlipg_batch_launch(mlipg_batch* b);
int mlipg_batch_compute(mlipg_batch* b, double* energies, double* forces, double* virials);
int mlipg_batch_results(mlipg_batch* b, double* energies, double* forces, double* virials);
size_t mlipg_batch_device_bytes(const mlipg_batch* b);
int mlipg_batch_sizes(const mlipg_batch* b, int* natoms, long long* npairs);
/* Autotunes the handle's tile shape on this batch (see mlipg_autotune). */
int mlipg_batch_autotune(mlipg_batch* b, int max_report, double* report, int* nreport);
void mlipg_batch_destroy(mlipg_batch* b);

/* Device neighbour lists for one or many periodic cells (no ghost atoms).
 * mlipg_dnlist_build wraps d_x4 (double4 x, y, z, element; cells stored one
 * after another, natoms[c] atoms each, lattice rows a1 a2 a3 per cell) into
 * its cells IN PLACE and builds full lists within rlist with packed image
 * codes ((n1+512) | (n2+512) << 10 | (n3+512) << 20, 0 for no shift): the
 * neighbour of i at entry p is x[idx[p]] + n1 a1 + n2 a2 + n3 a3.  Lists are
 * in a deterministic order (stencil bins, then atom index).  Pair arrays grow
 * with headroom_pct percent spare; mlipg_dnlist_arrays reports the device
 * arrays (CSR offsets, indices, image codes, cell of each atom, lattices),
 * the pair count, the longest list and a generation number that changes
 * whenever an array moved.  The reference builds its (half, displacement)
 * lists on the host: src/USER-MLIP/mlipkk_cell.cpp:218-307. */
typedef struct mlipg_dnlist mlipg_dnlist;
int mlipg_dnlist_create(void* cuda_stream, mlipg_dnlist** out);
int mlipg_dnlist_build(mlipg_dnlist* L, int ncells, const int* natoms, const double* lattices,
                       void* d_x4, double rlist, int headroom_pct);
int mlipg_dnlist_arrays(const mlipg_dnlist* L, const int** d_off, const int** d_idx,
                        const int** d_img, const int** d_center_cell, const double** d_cells,
                        long long* npairs, int* max_neigh, int* generation);
int mlipg_dnlist_copy(const mlipg_dnlist* L, int* off, int* idx, int* img);
void mlipg_dnlist_destroy(mlipg_dnlist* L);

/* Tile shape of the fused kernel and its autotuner.  No counterpart in the
 * reference (its Kokkos team sizes are fixed at compile time).
 * irr_chunk: coupling terms per batched work unit (even, 2..4096; default 24);
 * warp_order: 0 = units dealt round robin to the CTA's 8 warps in cost order,
 *             1 = longest first onto the least-loaded warp (one coupling order
 *                 at a time),
 *             2 = taken by the warps from a shared counter (order by order,
 *                 longest first);
 * ctas_per_sm: CTAs per SM of the persistent grid (0 = as many as fit).
 * Results agree between tilings to rounding (the energy summation is grouped
 * by unit).  mlipg_set_tiling waits for the handle's stream and re-uploads the
 * schedules; MD objects re-capture their step graph afterwards.
 * mlipg_autotune times every candidate (irr_chunk 12/24/48/96 x the three orders x
 * 1..resident CTAs/SM) on up to 16 centres per resident CTA of the given
 * structure (same arguments as mlipg_compute_device), keeps the fastest and
 * writes rows [irr_chunk, warp_order, ctas_per_sm, ms] to report (up to
 * max_report rows; *nreport = rows timed).  d_f and d_out8 are overwritten. */
int mlipg_set_tiling(mlipg_handle* h, int irr_chunk, int warp_order, int ctas_per_sm);
int mlipg_get_tiling(const mlipg_handle* h, int* out3);
int mlipg_autotune(mlipg_handle* h, int ncenters, const void* d_x4, const int* d_centers,
                   const int* d_nbr_off, const int* d_nbr_idx, const int* d_img,
                   const double* d_cell, const int* d_center_cell, int nb_cap, double* d_f,
                   double* d_out8, int max_report, double* report, int* nreport);

/* Serving: energy + force + stress requests for periodic structures of any
 * size, evaluated by continuous batching.  Requests (mlipg_server_submit,
 * thread-safe) are admitted in arrival order against a device-memory budget,
 * grouped by precision (MLIPG_PREC_FP64 or MLIPG_PREC_MIXED; other values are
 * MLIPG_EINVAL) into batches of at most max_batch_atoms atoms (FP64 batches:
 * at most min(max_batch_atoms, 8192) unless set by
 * mlipg_server_set_batch_atoms) and launched as they arrive; a precision
 * whose batch is full stops taking requests while the other precision is
 * still admitted in arrival order; FP64 and mixed batches run on separate
 * streams.
 * mlipg_server_wait returns a request's energy, forces[natoms*3] and virial
 * (LAMMPS order) or MLIPG_ETIMEDOUT at its deadline.  A request's energy
 * does not depend on the other requests in its batch.
 * mlipg_server_stats: [completed, p50 ms, p99 ms, atom-steps/s, batches,
 * device bytes in use, queued, in flight].  No counterpart in the reference. */
typedef struct mlipg_server mlipg_server;
int mlipg_server_create(const char* potential_path, size_t device_budget_bytes,
                        int max_batch_atoms, mlipg_server** out);
int mlipg_server_set_batch_atoms(mlipg_server* s, int precision, int max_atoms);
int mlipg_server_submit(mlipg_server* s, int natoms, const double* lattice9, const double* x,
                        const int* elements, int precision, long long* ticket);
int mlipg_server_wait(mlipg_server* s, long long ticket, int timeout_ms, double* energy,
                      double* forces, double* virial6);
int mlipg_server_stats(mlipg_server* s, double* out8);
void mlipg_server_destroy(mlipg_server* s);

/* NVE molecular dynamics on the device (velocity Verlet as LAMMPS `fix nve`,
 * metal units: A, ps, eV, g/mol; masses from the potential file).  Positions
 * x[natoms*3] and optional velocities v (A/ps) of one periodic cell
 * (lattice9 rows a1 a2 a3), elements 0-based; the full list is built with
 * cutoff + skin and rebuilt when an atom moves more than skin/2.  Each step
 * runs as one CUDA graph launch when use_graph is non-zero.  Reproduces the
 * trajectories of the reference's regression runs (fix nve,
 * the input scripts in test/regression); LAMMPS itself owns integration in
 * the drop-in path.
 * mlipg_md_thermo: [pe, ke, T (K), etotal, P, Pxx Pyy Pzz Pxy Pxz Pyz (bar),
 * list rebuilds], with dof = 3N - 3 as LAMMPS's thermo_temp. */
typedef struct mlipg_md mlipg_md;
int mlipg_md_create(mlipg_handle* h, const double* lattice9, int natoms, const double* x,
                    const double* v, const int* elements, double skin, mlipg_md** out);
int mlipg_md_run(mlipg_md* md, int nsteps, double dt_ps, int use_graph);
int mlipg_md_state(mlipg_md* md, double* x, double* v, double* f);
int mlipg_md_thermo(mlipg_md* md, double* out12);
/* Autotunes the handle's tile shape on this system (see mlipg_autotune) and
 * recomputes the forces at the current positions. */
int mlipg_md_autotune(mlipg_md* md, int max_report, double* report, int* nreport);
void mlipg_md_destroy(mlipg_md* md);

/* Training features of one periodic cell, the quantities a potential is
 * fitted to: its energy, forces and stress are linear in the regression
 * coefficients w (in the order of the potential file),
 *   E = sum_i polynomial[i] . w,  F_k = force[k] . w,  stress = stress . w.
 * Outputs (any may be NULL; host arrays):
 *   structural [natoms][n_structural]: the invariants d_{i,f}, feature index
 *     f = n * n_itc + itc as in the reference;
 *   polynomial [natoms][n_polynomial]: P_{i,p} = prod_{f in p} d_{i,f};
 *   force [natoms][n_polynomial][3]: the forces of E_p = sum_i P_{i,p}
 *     (F = force . w);
 *   stress [n_polynomial][6]: -sum over pairs r_ij (x) dE_p/dr_ij, order
 *     xx yy zz yz zx xy as the reference's stress features.
 * lattice9: cell vectors a1 a2 a3 as rows; x[natoms*3]; elements 0-based.
 * Evaluated in FP64 on the device (neighbour list built there).
 * Replaces MLIPModel::set_structure + prepare_features and the getters
 * get_structural_features / get_polynomial_features / get_force_features /
 * get_stress_features (src/USER-MLIP/mlipkk.cpp:278-372, 461-470, 992-1281,
 * 1322-1381).  mlipg_feature_sizes gives n_structural and n_polynomial. */
int mlipg_feature_sizes(const mlipg_handle* h, long long* n_structural, long long* n_polynomial);
int mlipg_features(mlipg_handle* h, int natoms, const double* lattice9, const double* x,
                   const int* elements, double* structural, double* polynomial, double* force,
                   double* stress);

/* Host neighbour-list builder for standalone and batched use: owned atoms
 * (wrapped into the cell), ghost images within `cutoff` in fractional
 * coordinates (LAMMPS's ghost rule for triclinic boxes), each atom's owner
 * and packed image code, and a full list (distance < cutoff) of the owned
 * atoms in CSR form.  lattice9 holds the cell vectors a1, a2, a3 as rows.
 * Replaces get_neighbors (src/USER-MLIP/mlipkk_cell.cpp:218-307), which
 * returns a half list of displacements instead. */
typedef struct mlipg_nlist mlipg_nlist;
int mlipg_nlist_build(const double* lattice9, int natoms, const double* x, const int* type,
                      double cutoff, mlipg_nlist** out);
int mlipg_nlist_sizes(const mlipg_nlist* nl, int* nall, long long* npairs);
int mlipg_nlist_copy(const mlipg_nlist* nl, double* x_all, int* type_all, int* owner,
                     int* image, int* nbr_off, int* nbr_idx);
void mlipg_nlist_destroy(mlipg_nlist* nl);

#ifdef __cplusplus
}
#endif

#endif /* MLIPG_H_ */
