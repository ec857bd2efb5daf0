/*
 * magace.h - C ABI of the GB300 implementation of the mag-ace potential
 * evaluation (non-collinear magnetic Atomic Cluster Expansion).
 *
 * Two layers:
 *
 *  1. The drop-in boundary. acelibini_ and acelib_ have exactly the symbol
 *     names and argument lists that the reference's LAMMPS pair style binds
 *     (lammps/pair_spin_ace.cpp:59-62) and that gfortran emits for the
 *     reference's Fortran entry points (src/ace.F90:10-21 and :79-107):
 *     lower-case name plus trailing underscore, every argument by reference,
 *     no hidden string lengths. A caller built against the reference links
 *     against libmagace.so unchanged. Like the reference they return nothing;
 *     where the reference would stop the process, this library records an
 *     error code (ace_last_error), prints one line to stderr and, for acelib_,
 *     fills the outputs with NaN.
 *
 *  2. The extended API (ace_*): explicit potential path, status codes,
 *     precision selection, and evaluation on device-resident arrays.
 *
 * All entry points serialise on one library-owned CUDA stream per process and
 * are not re-entrant (the reference keeps module-global state too).
 */
#ifndef MAGACE_H_
#define MAGACE_H_

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MAGACE_OK 0
#define MAGACE_ERR_FILE 1        /* potential file missing or unreadable */
#define MAGACE_ERR_FORMAT 2      /* malformed / inconsistent potential file */
#define MAGACE_ERR_UNSUPPORTED 3 /* nele != 1, radtype 0-2, nfemb 3/4, 5/6-body dims beyond the 3-body ones */
#define MAGACE_ERR_SMALL_R 4     /* bond shorter than one LUT bin (src/radial.F90:71-75) */
#define MAGACE_ERR_MOMENT 5      /* |m| < 0, NaN, or >= magnetic cutoff (LUT overrun in the reference) */
#define MAGACE_ERR_NOT_INIT 6    /* evaluation before a successful init */
#define MAGACE_ERR_ARGS 7        /* inconsistent arguments (ranges, element indices) */
#define MAGACE_ERR_CUDA 8        /* CUDA runtime failure (no device, out of memory, ...) */
#define MAGACE_ERR_NAN 9         /* non-finite density or energy */

/* ---- drop-in boundary (reference: src/ace.F90) -------------------------- */

/* Replaces acelibini (src/ace.F90:10-75). nele must be 1; elenumbers[0] is
 * the atomic number + 1 (the reference's element table starts with 'X',
 * lammps/pair_spin_ace.cpp:283-285). xcnumber 1 = pbe, 2 = lda. Reads
 * "<El>.<xc>.in" from the current working directory (src/util.F90:525).
 * Idempotent after the first success (src/util.F90:29-33). */
void acelibini_(int* nele, double* rcut, double* rcut_magnetic, double* smear, int* xcnumber,
                int* elenumbers);

/* Replaces acelib (src/ace.F90:79-321). Inputs (caller-owned, read-only):
 *   nlist[nei] 1-based j (unused), occ[natom], occlist[nei] (must be 1),
 *   nstart/nstop[natom] 1-based inclusive bond ranges,
 *   dlist[nei] = r_ij, elist[3*nei] = (x_i - x_j)/r_ij,
 *   dlist_momi[natom] = |m_i|, elist_momi[3*natom] = m_hat_i,
 *   dlist_mom[nei] = |m_j|, elist_mom[3*nei] = m_hat_j.
 * Outputs: eout[natom] = E_i; flist[3*nei] = dE_i/d(x_i - x_j) per bond;
 *   tlist[3*nei] = dE_i/dm_j per bond; tlist0[3*natom] = dE_i/dm_i.
 *   Per-bond outputs are packed atom by atom in bond order
 *   (src/ace.F90:291-318). Computed on the GPU in the precision selected by
 *   ace_set_precision (default: FP64). */
void acelib_(int* natom, int* nall, int* nei, int* nlist, int* occ, int* occlist, int* nstart,
             int* nstop, double* eout, double* dlist, double* elist, double* flist,
             double* dlist_momi, double* elist_momi, double* dlist_mom, double* elist_mom,
             double* tlist, double* tlist0);

/* ---- status (no counterpart in the reference, which stops instead) ----- */
int ace_last_error(void);
const char* ace_error_string(int code);
const char* ace_last_error_message(void);
void ace_clear_error(void);

/* ---- extended API -------------------------------------------------------- */

/* As acelibini_ but with an explicit file path and element symbol; replaces
 * any previous potential. Host-only: builds every table but touches no GPU. */
int ace_init_file(const char* path, const char* element, double rcut, double rcut_magnetic,
                  double smear, int xcnumber);

/* 0 = FP64 (the drop-in default, parity <= 1e-10 relative, bitwise
 *     reproducible): features, densities, embedding and outputs in double;
 *     with the specialised kernels the contractions run as compensated
 *     float-float dot products (48-bit operands, about 1e-14 from FP64).
 * 1 = split precision: FP32 basis/products with FP64 accumulation of the
 *     per-atom energy and the embedding near zero density. */
int ace_set_precision(int mode);
int ace_get_precision(void);

/* Basis sizes after init: out[0..3] = number of 1-,2-,3-,4-body clusters
 * (nvar1..nvar4), out[4..6] = 2-,3-,4-body product terms, out[7] = cluster
 * records in the file that matched no enumerated cluster. */
int ace_basis_sizes(int* out);

/* Cluster index rows as in the file's 'clu' records: rank 1 -> 1 int per
 * cluster, 2 -> 4, 3 -> 9, 4 -> 15, 5 -> 21, 6 -> 27 (the reference's
 * b5index / b6index, src/util.F90:2817-3760). */
int ace_basis_rows(int rank, int* out);

/* Number of clusters of one rank (1..6) after init (nvar1..nvar6 of the
 * reference, src/util.F90:1613-3760); sizes the ace_basis_rows output. */
int ace_basis_count(int rank, int* count);

/* Evaluation on device-resident arrays (no host copies). Bonds of atom i are
 * bond_offset[i] .. bond_offset[i+1]-1 (0-based CSR, natom+1 entries).
 * r[nei], e[3*nei] = (x_i - x_j)/r, mag_j[nei], mhat_j[3*nei], mag_i[natom],
 * mhat_i[3*natom]; outputs energy[natom], fij[3*nei], tij[3*nei], ti0[3*natom].
 * `stream` is a cudaStream_t or NULL for the library's own stream, which is
 * non-blocking: it does not wait for work on other streams, so a caller
 * whose inputs are still being written on another stream passes that stream
 * (cudaStreamLegacy for the legacy default stream) or synchronises first. The call is
 * asynchronous with respect to the host. Check ace_device_status() after the
 * stream has completed. One call (this one, ace_descriptors_device and acelib_)
 * takes at most 715,827,882 bonds and atoms, since the kernels index the
 * per-bond vectors as 3 j with 32-bit j; larger calls are refused with
 * MAGACE_ERR_ARGS. */
int ace_compute_device(int natom, int nei, const int* bond_offset, const double* r,
                       const double* e, const double* mag_j, const double* mhat_j,
                       const double* mag_i, const double* mhat_i, double* energy, double* fij,
                       double* tij, double* ti0, void* stream);

/* Reads (and clears) the device-side error word of the last ace_compute_device
 * call; synchronises the library stream. */
int ace_device_status(void);

/* How acelib_ reaches the caller's host arrays on the current device:
 * 0 = pageable copies, 1 = staged through pinned memory, 2 = the kernels read
 * and write the caller's memory directly (the GPU uses the host page tables,
 * as with NVLink-C2C on Grace). The environment variable MAGACE_HOST_ACCESS
 * (copy | pinned | direct | auto) chooses; "auto" (default) takes 2 when the
 * device supports it, else 1. Returns -1 when no tables could be placed. */
int ace_host_access_mode(void);

/* Number of kernels launched by the last evaluation call: 5 for the
 * specialised (example Fe) layout in either precision (A basis, 2-/4-body
 * density, 3-body density, k_finish_fe, forces), 3 for the generic kernels
 * of other layouts (A basis, density, forces). */
int ace_last_launch_count(void);

/* Kernel timing: when on, the boundaries of the kernels of every evaluation
 * are recorded with CUDA events on the evaluation stream, and every kernel
 * runs on that stream (the specialised layout otherwise runs its 2-/4-body
 * and 3-body density kernels side by side on two streams); ace_kernel_times
 * writes the last evaluation's per-kernel durations in ms into ms[0..3],
 * synchronising on the last event: k_abasis, k_density, k_b3 (with
 * k_finish_fe), k_forces (specialised layout, either precision), or
 * k_abasis, k_density, k_forces (generic kernels). Entries beyond those are
 * 0. */
int ace_set_kernel_timing(int on);
int ace_kernel_times(float* ms);

/* Gather-table statistics: out[0..2] entries with 1/2/3 other factors,
 * out[3] segments, out[4] output slots, out[5] factors per atom (nF),
 * out[6] weights per atom (nW), out[7] A weight slots, out[8] A2 half slots,
 * out[9] atomic LUT functions, out[10] magnetic LUT functions, out[11..20]
 * the basis dims nradbase_a, nradbase_m, nradial2_m, l2max_m, nradial3_a,
 * nradial3_m, l3max_a, l3max_m, and the half-plane sizes h2, h3;
 * out[21..25] the dense 3-body tables of the specialised kernels: tasks,
 * angular combinations, half-plane elements, and the segments and entries of
 * the remaining (non-3-body) gather table; out[26..28] that table's entries
 * by arity 1..3; out[29] the coefficient pairs the dense 3-body contraction
 * visits per atom; out[30] the factors that table reads (31 entries). */
int ace_table_stats(long long* out);

/* Allocation-free variant of ace_compute_device, for callers that cannot
 * allocate device memory when they evaluate (an allocator they do not own,
 * MD drivers that forbid allocation after set-up). It has no counterpart in
 * the reference. Same arguments and results as ace_compute_device, but it
 * calls no cudaMalloc/cudaFree or allocating routine: its per-atom scratch
 * lives in one fixed 64 MiB device array that every GPU loading the library
 * holds until exit, which bounds natom: for the example Fe basis on a
 * 152-SM GB300, at most 1,816 atoms in FP64 and 3,305 in the split precision
 * (the refusal's message gives the limit for the loaded potential). Larger
 * calls, and calls beyond ace_compute_device's bond limit, are refused with
 * MAGACE_ERR_ARGS. When the bond arrays are device memory, the A-basis
 * kernel variants that stage bond tiles with bulk copies may run, as in
 * ace_compute_device. The potential's tables must already be on the device
 * (placed by any ace_compute_device call; natom = 0 is enough). The first call
 * on each device looks up the scratch address (cudaGetSymbolAddress). Calls
 * share the scratch, so calls that overlap on the GPU race. The call is
 * synchronous: it returns after the evaluation has completed, with this
 * call's device-side status, so it cannot be captured into a CUDA graph; on a
 * stream that is capturing it returns MAGACE_ERR_ARGS before any device work. */
int ace_compute_device_noalloc(int natom, int nei, const int* bond_offset, const double* r,
                               const double* e, const double* mag_j, const double* mhat_j,
                               const double* mag_i, const double* mhat_i, double* energy,
                               double* fij, double* tij, double* ti0, void* stream);

/* Work queue (no counterpart in the reference): with on != 0, every
 * evaluation first sorts its atoms by decreasing bond count on the device
 * (three small kernels) and the persistent kernels take the atoms in that
 * order: a longest-first schedule for batches of configurations of uneven
 * size and neighbour count. Results do not change. Off by default;
 * ace_compute_device_noalloc always uses the natural order. */
int ace_set_work_queue(int on);

/* Autotuner (no counterpart in the reference): evaluates the given system
 * (same arrays as ace_compute_device) with every variant of the
 * split-precision kernels (CTA shapes of the A-basis, 2-/4-body and 3-body
 * density kernels; the force kernel's CTAs per SM and its FP32 or
 * tensor-core form), times each kernel with CUDA events and keeps each
 * kernel's fastest variant for later evaluations. Writes the choices.
 * Synchronous. Results change only within FP32 rounding (the 3-body sums'
 * order; the tensor-core products' 3xTF32 split, below 2^-20 relative). For
 * the FP64 path or another basis layout it only reports the current choice. */
int ace_autotune_device(int natom, int nei, const int* bond_offset, const double* r, const double* e,
                        const double* mag_j, const double* mhat_j, const double* mag_i,
                        const double* mhat_i, void* stream, int* rest_warps, int* b3_warps,
                        int* force_blocks);

/* The kernel variants in use, variants[4]: A basis (0 scalar, 1 packed
 * FP32x2, 2 scalar with the bond tiles staged into shared memory by TMA bulk
 * copies, 3 the same on a persistent grid, 4 the bond sums on the tensor
 * cores with 3's staging, 5 the tensor-core sums alone; 2-4 run only when the
 * bond arrays are device memory and otherwise fall back to 0 (2, 3) or 5 (4)), 2-/4-body density (0/1: 32/16 warps with per-entry loads, 2/3:
 * 32/16 warps reading record streams by shuffles, 4/5: through shared
 * memory), 3-body (0-2: 16/12/8 warps, 3: 12
 * warps with the n0' loop outermost, 4/5: 16/12 warps packed FP32x2), forces
 * (0-2: 4/6/8 CTAs per SM, 3-5: the same packed FP32x2, 6/7: 5/6 CTAs per SM
 * with the contractions as GEMMs on the tensor cores, mma.sync TF32 in the
 * 3xTF32 split). Until the autotuner or ace_set_tuning chooses, the variants
 * are {4, 4, 4, 6}, the fastest on a 15,840-atom bcc Fe workload. */
int ace_get_tuning(int* variants);

/* Selects the kernel variants directly (no counterpart in the reference):
 * variants[4] as ace_get_tuning reports them; an index out of a kernel's
 * range is an error (MAGACE_ERR_ARGS). Results change only within FP32
 * rounding (the 3-body sums' order, the tensor-core products' split). */
int ace_set_tuning(const int* variants);

/* ---- Differentiation and fitting (no counterpart in the reference's
 * acelib_; they expose what src/forces.F90:976-1289 computes internally). ----
 *
 * The expansion coefficients as one vector c[ndensity][ncoef]: the 'clu'
 * records of ranks 1..4 in the file's order (ace_basis_rows). The density
 * of atom i is rho_d = sum_k c[d][k] B_k(i). */
int ace_num_coefficients(int* ncoef, int* ndensity);
int ace_get_coefficients(double* c);
/* Replaces the coefficients and rebuilds the tables that fold them in; the
 * next device call uploads them. */
int ace_set_coefficients(const double* c);

/* Descriptors B[natom][ncoef] (FP64) of the atoms described by the same
 * device arrays as ace_compute_device: rank 1, g_n(|m_i|) - 1; ranks 2..4,
 * the basis functions of src/b_basis.F90:91-307 without their coefficients.
 * Asynchronous on `stream`. With dE_i/drho_d from
 * ace_density_gradient_device, dE_i/dc[d][k] = dE_i/drho_d * B_k(i). */
int ace_descriptors_device(int natom, int nei, const int* bond_offset, const double* r,
                           const double* e, const double* mag_j, const double* mhat_j,
                           const double* mag_i, const double* mhat_i, double* B, void* stream);

/* Descriptors and their directional derivatives, for the coefficient
 * gradients of losses on forces and magnetic forces (fitting). Along the
 * tangents dd[3*nei] of the bond vectors x_i - x_j (dd_ij = u_i - u_j for a
 * displacement field u), dm_j[3*nei] of the neighbours' moments and
 * dm_i[3*natom] of the atoms' own moments, writes B[natom][ncoef] (as
 * ace_descriptors_device), Bdot[natom][ncoef] = dB/d(epsilon) at epsilon = 0
 * of the inputs moved by epsilon times the tangents, and the core energy
 * core[natom] and its derivative core_dot[natom]. FP64, asynchronous on
 * `stream`; the other arguments as ace_compute_device. No counterpart in the
 * reference, whose fitting code is not part of it (src/Makefile:107-108). */
int ace_descriptors_tangent_device(int natom, int nei, const int* bond_offset, const double* r,
                                   const double* e, const double* mag_j, const double* mhat_j,
                                   const double* mag_i, const double* mhat_i, const double* dd,
                                   const double* dm_j, const double* dm_i, double* B, double* Bdot,
                                   double* core, double* core_dot, void* stream);

/* The embedding of the loaded potential (src/forces.F90:1134-1266): nfemb,
 * par[2*order + density] (order 0: prefactor, 1: exponent; density 0, 1),
 * and the inner cutoff inner_cutoff[0..1] = ecut, decut on the core energy
 * (src/forces.F90:1112-1128). Any pointer may be NULL. */
int ace_embedding(int* nfemb, double* par, double* inner_cutoff);

/* Copies dE_i/drho_d [natom][2] (d = 0, 1; the second is 0 for one density)
 * of the last ace_compute_device or acelib_ evaluation into a device array,
 * on `stream`. */
int ace_density_gradient_device(int natom, double* dedrho, void* stream);

/* ---- Spin-lattice molecular dynamics on the device (no counterpart in
 * the reference, which is driven by LAMMPS fix nve/spin). ----
 *
 * One configuration of natom atoms: positions x[3*natom] (A), velocities
 * v[3*natom] (A/ps), moments m[3*natom] (mu_B, Cartesian), cell[9] (rows are
 * lattice vectors, A), pbc[3]; mass in amu; bonds listed within rcut + skin.
 * A periodic axis must be at least 3 (rcut + skin) wide. Returns a handle. */
int ace_md_create(int natom, const double* x, const double* v, const double* m, const double* cell,
                  const int* pbc, double mass_amu, double rcut, double skin, int* handle);
/* nsteps steps of dt_ps: v += dt/2 F/m; x += dt v; every moment turns about
 * its field fm = -(mub/hbar) dE/dm by |fm| dt (|m| kept); forces and fields
 * at the new state; v += dt/2 F/m. The neighbour list is rebuilt every
 * rebuild_every steps; with use_graph the steps in between replay one
 * captured CUDA graph. log[2*(nsteps+1)] (may be NULL) receives the total
 * potential and kinetic energy (eV) of the start and after every step. The
 * evaluation uses the current precision (ace_set_precision). */
int ace_md_run(int handle, int nsteps, double dt_ps, int rebuild_every, int use_graph, double* log);
/* Copies the state to host arrays of 3*natom doubles (any may be NULL):
 * positions, velocities, moments, forces -dE/dx and fields fm. */
int ace_md_state(int handle, double* x, double* v, double* m, double* F, double* fm);
/* The current neighbour list: nbond, off[natom+1], j[nbond], image shift
 * (three bytes biased by 128) and the index of each bond's reverse. */
int ace_md_bonds(int handle, int* nbond, int* off, int* j, int* shift, int* rev);
int ace_md_destroy(int handle);

/* Releases every device buffer held by the library (tables stay on the host). */
void ace_release_device(void);

#ifdef __cplusplus
}
#endif

#endif /* MAGACE_H_ */
