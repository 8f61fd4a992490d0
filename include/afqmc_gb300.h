/*
 * afqmc_gb300.h - C ABI of the GB300-native phaseless-AFQMC hot path.
 *
 * The reference (zh-yichi/cs_afqmc, package ad_afqmc) is pure Python on JAX and has no
 * foreign-function layer of its own: its hot path is a set of jitted Python methods. Each
 * entry point below replaces one of those methods, cited as file:line inside ad_afqmc/.
 * A Python host (cs_afqmc_gb300, via ctypes) or any C caller binds them.
 *
 * Conventions
 *  - All array arguments are DEVICE pointers owned by the caller, row-major, with complex
 *    numbers stored interleaved (re, im). No function allocates device memory except where
 *    stated; scratch lives in the caller-provided workspace (afq_workspace_size).
 *  - Every call is stream-ordered on the caller's cudaStream_t (passed as void*), performs
 *    no host synchronisation and is capturable into a CUDA graph.
 *  - Return value: 0 on success; negative on a host-side error (bad shape, pointer or
 *    unsupported option: nothing was launched); positive on a CUDA launch error.
 *    afq_last_error() returns a message for the last failure on the calling thread.
 *  - A context is not thread-safe; several contexts may share one device.
 *
 * Walker containers mirror the reference (wavefunctions.py:15-43):
 *  - restricted walkers: one slab [nw, norb, max(n_up, n_dn)];
 *  - unrestricted walkers: two slabs [nw, norb, n_up] and [nw, norb, n_dn].
 * Walker element type: complex128 when precision == AFQ_PREC_FP64, complex64 when
 * precision == AFQ_PREC_MIXED.
 */
#ifndef AFQMC_GB300_H
#define AFQMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AFQ_ABI_VERSION 1

enum afq_walker_type { AFQ_WALKERS_RESTRICTED = 0, AFQ_WALKERS_UNRESTRICTED = 1 };
enum afq_trial_type { AFQ_TRIAL_RHF = 0, AFQ_TRIAL_UHF = 1 };
enum afq_precision {
  AFQ_PREC_FP64 = 0,  /* every contraction in FP64 (the reference's arithmetic) */
  AFQ_PREC_MIXED = 1  /* BF16 tensor-core contractions with split-BF16 correction, FP32
                         walkers, FP64 determinants / weights / energy accumulation */
};

/* Sizes and options. Mirrors the static fields of the reference's dataclasses:
 * propagator_restricted(dt, n_walkers, n_exp_terms, n_batch) (propagation.py:201-212) and
 * rhf/uhf(norb, nelec) (wavefunctions.py:453-476, 638-660). */
typedef struct afq_dims {
  int32_t norb;
  int32_t n_up;
  int32_t n_dn;
  int32_t nchol;
  int32_t n_walkers;
  int32_t walker_type;  /* afq_walker_type */
  int32_t trial_type;   /* afq_trial_type */
  int32_t precision;    /* afq_precision */
  int32_t n_exp_terms;  /* Taylor terms of exp(vhs), reference default 6 */
  int32_t n_batch;      /* walker chunks for the vhs workspace (>= 1, divides n_walkers) */
  int32_t mixed_config; /* AFQ_PREC_MIXED accuracy options; 0 = library default (767).
                           bits 0..7: lo (correction) terms of G / rot_chol (force bias),
                           fields / chol (vhs), walker / exp_h1 (exp_h1 products), G /
                           rot_chol (energy); bits 8..10: Taylor products with split
                           operands; bit 11: bf16 instead of fp16; bits 12..14: K tiles per
                           drained accumulation run of the force-bias, vhs and exchange
                           GEMMs (0 = default, 7 = undrained); bit 15: every Cholesky
                           vector is a diagonal matrix (on-site lattice terms), so exp(vhs)
                           W1 is a per-row polynomial scale and the vhs GEMM and Taylor
                           products are skipped (checked on the device: an off-diagonal
                           nonzero ors 4 into scalars[AFQ_S_STATUS]) */
  double dt;
} afq_dims;

/* Hamiltonian and trial intermediates built by hamiltonian.build_measurement_intermediates
 * and build_propagation_intermediates (hamiltonian.py:49-81 -> wavefunctions.py:602-619,
 * 817-841; propagation.py:292-325, 464-509). Device pointers; the caller keeps them alive
 * for the context's lifetime. The trial must be real (float64 mo_coeff). */
typedef struct afq_hamiltonian {
  double h0;
  double h0_prop_re, h0_prop_im;  /* -h0 - sum(mf_shifts^2)/2 */
  const double* trial_up;         /* [norb, n_up] mo_coeff (spin up; RHF: the only one) */
  const double* trial_dn;         /* [norb, n_dn] (UHF); NULL for RHF */
  const double* chol;             /* [nchol, norb*norb] */
  const double* rot_chol_up;      /* [nchol, n_up, norb]  C_up^H L_g */
  const double* rot_chol_dn;      /* [nchol, n_dn, norb]  (UHF); NULL for RHF */
  const double* rot_h1_up;        /* [n_up, norb] */
  const double* rot_h1_dn;        /* [n_dn, norb] (UHF); NULL for RHF */
  const double* exp_h1_up;        /* [norb, norb] expm(-dt h1_mod/2) */
  const double* exp_h1_dn;        /* [norb, norb] (unrestricted walkers); NULL otherwise */
  const double* mf_shifts;        /* [nchol] complex128 */
} afq_hamiltonian;

/* Propagation state, the device-resident part of the reference's prop_data dict
 * (propagation.py:210-232). scalars[] indices below. */
typedef struct afq_walker_state {
  void* walkers_up;   /* restricted: the only slab */
  void* walkers_dn;   /* unrestricted only */
  double* weights;    /* [nw] */
  double* overlaps;   /* [nw] complex128 */
  double* scalars;    /* [AFQ_NSCALARS] */
} afq_walker_state;

enum afq_scalar_index {
  AFQ_S_E_ESTIMATE = 0,        /* prop_data["e_estimate"] */
  AFQ_S_POP_CONTROL_SHIFT = 1, /* prop_data["pop_control_ene_shift"] */
  AFQ_S_N_KILLED = 2,          /* prop_data["n_killed_walkers"] */
  AFQ_S_BLOCK_ENERGY = 3,      /* last block's weighted energy */
  AFQ_S_BLOCK_WEIGHT = 4,      /* last block's total weight */
  AFQ_S_STATUS = 5,            /* device-side guard word (0 = ok) */
  AFQ_NSCALARS = 8
};

typedef struct afq_ctx afq_ctx;

/* ---- context ------------------------------------------------------------------------ */

/* Bytes of device workspace a context with these sizes needs. Returns 0 on bad sizes. */
size_t afq_workspace_size(const afq_dims* dims);

/* Create a context. `workspace` must hold afq_workspace_size(dims) bytes (256-B aligned)
 * and stays owned by the caller. Converts and caches precision-specific copies of the
 * Hamiltonian inside the workspace (stream-ordered on `stream`). */
int afq_ctx_create(const afq_dims* dims, const afq_hamiltonian* ham, void* workspace,
                   size_t workspace_bytes, void* stream, afq_ctx** out);
void afq_ctx_destroy(afq_ctx* ctx);
const char* afq_last_error(void);
int afq_abi_version(void);

/* ---- trial measurements (wave_function.calc_*) --------------------------------------- */

/* Overlap <psi_T|walker> per walker, complex128 [nw].
 * Replaces wave_function.calc_overlap, wavefunctions.py:45-96 (rhf 478-488, uhf 658-667). */
int afq_calc_overlap(afq_ctx* ctx, const void* walkers_up, const void* walkers_dn,
                     double* overlaps, void* stream);

/* Force bias <psi_T|L_g|walker>/<psi_T|walker>, complex128 [nw, nchol].
 * Replaces wave_function.calc_force_bias, wavefunctions.py:111-165 (rhf 503-527,
 * uhf 694-709). */
int afq_calc_force_bias(afq_ctx* ctx, const void* walkers_up, const void* walkers_dn,
                        double* force_bias, void* stream);

/* Mixed local energy, complex128 [nw].
 * Replaces wave_function.calc_energy, wavefunctions.py:186-241 (rhf 529-561,
 * uhf 711-743). */
int afq_calc_energy(afq_ctx* ctx, const void* walkers_up, const void* walkers_dn,
                    double* energies, void* stream);

/* ---- propagator ---------------------------------------------------------------------- */

/* One phaseless step with the given fields (float64 [nw, nchol]): force bias, shifted
 * fields, exp(vhs) by Taylor series between two exp_h1 half steps, new overlaps,
 * phaseless importance function and clamps, weights and pop_control_ene_shift.
 * Replaces propagator.propagate, propagation.py:100-165 (+ _apply_trotprop 255-290,
 * 359-400 and _apply_trotprop_det 67-92). */
int afq_propagate(afq_ctx* ctx, afq_walker_state* state, const double* fields, void* stream);

/* Q of the reduced QR of every walker slab (LAPACK Householder convention in FP64 mode).
 * Replaces propagator.orthonormalize_walkers, propagation.py:251-253, 422-424
 * (linalg_utils.py:51-65). */
int afq_orthonormalize_walkers(afq_ctx* ctx, afq_walker_state* state, void* stream);

/* Comb stochastic reconfiguration with uniform *zeta (device pointer). Writes the chosen
 * source index per walker to `indices` (int32 [nw], may be NULL).
 * Replaces sr.stochastic_reconfiguration(_uhf), sr.py:24-47, as called by
 * propagator.stochastic_reconfiguration_local, propagation.py:234-240, 402-408. */
int afq_stochastic_reconfiguration(afq_ctx* ctx, afq_walker_state* state, const double* zeta,
                                   int32_t* indices, void* stream);

/* ---- sampler ------------------------------------------------------------------------- */

/* sampler.propagate_phaseless, sampling.py:319-341 (with _sr_block_scan 126-144 and
 * _block_scan 50-92): n_sr_blocks x [n_ene_blocks x [n_prop_steps propagate, QR,
 * overlaps, clamped energies, block energy/weight, pop-control update], local SR].
 * fields: float64 [n_sr_blocks, n_ene_blocks, n_prop_steps, nw, nchol];
 * zetas: float64 [n_sr_blocks]; block_energy / block_weight: float64
 * [n_sr_blocks * n_ene_blocks]; energy: float64 [1] = sum(E_b w_b)/sum(w_b).
 * All on the device; no host synchronisation. */
int afq_propagate_phaseless(afq_ctx* ctx, afq_walker_state* state, const double* fields,
                            const double* zetas, int32_t n_prop_steps, int32_t n_ene_blocks,
                            int32_t n_sr_blocks, double* block_energy, double* block_weight,
                            double* energy, void* stream);

/* Per-block driver bookkeeping for one rank (driver.py:250-308, non-AD branch):
 * *block_weight = sum(weights) (before QR/SR), e_estimate <- 0.9 e_estimate + 0.1 *energy,
 * QR of every walker, then the comb SR with uniform *zeta (the single-rank
 * stochastic_reconfiguration_global, sr.py:66-106). energy, zeta, block_weight are device
 * pointers to one double each. */
int afq_block_end(afq_ctx* ctx, afq_walker_state* state, const double* energy, const double* zeta,
                  double* block_weight, void* stream);

/* ---- free projection (FP64, unrestricted walkers) ------------------------------------ */

/* One free-projection step with unshifted fields (float64 [nw, nchol]): no force bias, no
 * phaseless constraint. Each slab s times exp(-sqrt(dt) sum_g x_g mf_g / (2 n_s))
 * exp(dt (h0_prop + ene0) / (2 n_s)) after exp(vhs) between the exp_h1 half steps; QR of both
 * slabs with norms (complex128 [nw]) *= prod(diag R_up) prod(diag R_dn); state->overlaps =
 * overlap of the new walkers * norms; normed_overlaps (complex128 [nw]) = overlap of the walkers
 * QR-ed once more. Replaces propagator_unrestricted.propagate_free (propagation.py:436-462,
 * intermediates 464-490). Weights and scalars are not used. */
int afq_propagate_free(afq_ctx* ctx, afq_walker_state* state, const double* fields, double ene0,
                       double* norms, double* normed_overlaps, void* stream);

/* n_blocks free-projection blocks of n_prop_steps steps (fields float64
 * [n_blocks, n_prop_steps, nw, nchol]), starting from state->overlaps = overlap(walkers):
 * after each block the complex local energies E and block_energy[b] = sum E O / sum O,
 * block_weight[b] = sum O (complex128 [n_blocks], O = state->overlaps). Replaces
 * sampler.propagate_free / _block_scan_free (sampling.py:95-124, 344-360); the per-block
 * prop_data trajectory the reference returns is not kept. */
int afq_propagate_free_blocks(afq_ctx* ctx, afq_walker_state* state, const double* fields,
                              int32_t n_prop_steps, int32_t n_blocks, double ene0, double* norms,
                              double* normed_overlaps, double* block_energy,
                              double* block_weight, void* stream);

/* ---- CPMC, Hubbard model with on-site U (FP64, real walkers) ------------------------- */

/* Overlaps det(C_up^T W_up) det(C_dn^T W_dn) (float64 [nw]) and full Green's functions
 * greens (float64 [nw][2][norb][norb], G_s = (W_s (C_s^T W_s)^-1 C_s^T)^T) of real walkers
 * ([nw][norb][n_up], [nw][norb][n_dn]) for the real UHF trial C_up [norb, n_up], C_dn
 * [norb, n_dn]: the part of propagator_cpmc.init_prop_data that needs the walkers
 * (propagation.py:518-537, uhf_cpmc.calc_full_green wavefunctions.py:894-914). No context;
 * norb <= 64, n_up, n_dn <= 32. */
int afq_cpmc_init(int32_t norb, int32_t n_up, int32_t n_dn, int32_t n_walkers,
                  const double* trial_up, const double* trial_dn, double* walkers_up,
                  double* walkers_dn, double* overlaps, double* greens, void* stream);

/* One CPMC step (propagator_cpmc.propagate, propagation.py:565-657): exp_h1 half step with
 * the overlap-ratio weight update (weights < 1e-8 -> 0), then for every site x a discrete
 * Hubbard-Stratonovich field, field f chosen with probability proportional to
 * (1 + (c_f,up - 1) G_up[x,x]) (1 + (c_f,dn - 1) G_dn[x,x]) (ratios < 1e-8 -> 0; uniforms
 * (erf(g / sqrt 2) + 1) / 2 of gaussian [nw][norb]), c = exp(-dt u / 2) exp(+-gamma),
 * cosh(gamma) = exp(dt u / 2); walker rows x scaled, rank-one Green's-function updates
 * (wavefunctions.py:916-945), overlaps * ratio, weights * normalisation; exp_h1 half step;
 * weights * exp(dt pop_control_ene_shift), > 100 -> 0; scalars[AFQ_S_POP_CONTROL_SHIFT] =
 * e_estimate - 0.1 log(sum w / nw) / dt. exp_h1_up / exp_h1_dn: float64 [norb, norb].
 * greens as in afq_cpmc_init, updated. */
int afq_cpmc_propagate(int32_t norb, int32_t n_up, int32_t n_dn, int32_t n_walkers, double dt,
                       double u, const double* exp_h1_up, const double* exp_h1_dn,
                       const double* trial_up, const double* trial_dn, double* walkers_up,
                       double* walkers_dn, double* weights, double* overlaps, double* greens,
                       double* scalars, const double* gaussian, void* stream);

/* One step of the continuous-field CPMC variant (propagator_cpmc_continuous,
 * propagation.py:1595-1675, whose force bias is multiplied by zero): exp_h1 half step; rows i
 * of the up / down slab times exp(+x_i hs_constant) / exp(-x_i hs_constant) with the
 * Gaussians x = gaussian[w] (float64 [nw][norb]); exp_h1 half step; weights *=
 * exp(dt pop_control_ene_shift) O'/O (< 1e-8 -> 0, > 100 -> 0); overlaps = O'; then the
 * pop-control shift as in afq_cpmc_propagate. Real walkers, no Green's functions. */
int afq_cpmc_continuous_propagate(int32_t norb, int32_t n_up, int32_t n_dn, int32_t n_walkers,
                                  double dt, double hs_constant, const double* exp_h1_up,
                                  const double* exp_h1_dn, const double* trial_up,
                                  const double* trial_dn, double* walkers_up, double* walkers_dn,
                                  double* weights, double* overlaps, double* scalars,
                                  const double* gaussian, void* stream);

/* One CPMC step with on-site U and a nearest-neighbour interaction u_1 (propagator_cpmc_nn,
 * propagation.py:889-1230): one-body half step, the on-site sweep of
 * afq_cpmc_propagate, then for every neighbour pair (i, j) four two-entry updates with the
 * Hubbard-Stratonovich constants of u_1 on (up i, up j), (up i, dn j), (dn i, up j),
 * (dn i, dn j), one-body half step, weights * exp(dt shift), the > 100 clamp and the new
 * pop-control shift. neighbors: device int32 [n_pairs][2], sites in [0, norb), i != j (a
 * bad pair is skipped and sets scalars[AFQ_S_STATUS] = 3). uniforms: device float64
 * [n_walkers][norb + 4 n_pairs], column x for site x, then column norb + k n_pairs + p for
 * update k of pair p (the reference draws both sets from its key). The two-entry updates
 * within one spin use the exact rank-two Green's-function update. Other arguments as in
 * afq_cpmc_propagate. */
int afq_cpmc_nn_propagate(int32_t norb, int32_t n_up, int32_t n_dn, int32_t n_walkers, double dt, double u,
                          double u_1, const int32_t* neighbors, int32_t n_pairs, const double* exp_h1_up,
                          const double* exp_h1_dn, const double* trial_up, const double* trial_dn,
                          double* walkers_up, double* walkers_dn, double* weights, double* overlaps,
                          double* greens, double* scalars, const double* uniforms, void* stream);

/* ---- forward-mode derivative of the block (differentiation pattern, FP64) ------------ */

/* Bytes of device tangent workspace afq_propagate_phaseless_jvp needs. 0 on bad sizes. */
size_t afq_tangent_workspace_size(const afq_dims* dims);

/* flags of afq_propagate_phaseless_jvp and afq_propagate_phaseless_vjp */
enum {
  AFQ_JVP_NO_SR = 1 /* no local SR after the energy blocks (the _nosr variants,
                       sampling.py:221-254, 287-317); needs n_sr_blocks == 1, zetas may be NULL */
};

/* afq_propagate_phaseless together with its derivative with respect to a coupling lambda of
 * h1 + lambda * D, the trial held fixed: the jvp that driver.py:207-215 takes of
 * sampler.propagate_phaseless_ad_norot (sampling.py:266-285) with tangent 1 on the
 * coupling and zero on prop_data. The only inputs with a tangent are the propagator's
 * exp_h1 and the measurement intermediate rot_h1, whose derivatives the caller passes:
 * dexp_h1_up/dn float64 [norb, norb] (d expm(-dt h1_mod/2) / d lambda; dn NULL for
 * restricted walkers) and drot_h1_up/dn with the layout of rot_h1_up/dn (dn NULL for the
 * RHF trial). Values (walkers, weights, overlaps, scalars, block_energy, block_weight,
 * energy) are those of afq_propagate_phaseless on the same draws; dblock_energy,
 * dblock_weight ([n_sr_blocks * n_ene_blocks]) and denergy ([1]) are their derivatives.
 * Clamped quantities (weights set to 0, local energies replaced by e_estimate) have a zero
 * derivative, as jnp.where's jvp gives. tangent_workspace: 256-B aligned device memory of
 * afq_tangent_workspace_size(dims) bytes, cleared by the call. FP64 contexts only. */
int afq_propagate_phaseless_jvp(afq_ctx* ctx, afq_walker_state* state, const double* dexp_h1_up,
                                const double* dexp_h1_dn, const double* drot_h1_up,
                                const double* drot_h1_dn, void* tangent_workspace,
                                size_t tangent_workspace_bytes, const double* fields,
                                const double* zetas, int32_t n_prop_steps, int32_t n_ene_blocks,
                                int32_t n_sr_blocks, int32_t flags, double* block_energy,
                                double* block_weight, double* dblock_energy,
                                double* dblock_weight, double* energy, double* denergy,
                                void* stream);

/* Tangent inputs of afq_propagate_phaseless_jvp_ex (device float64 arrays, NULL where not
 * applicable). dexp_h1 / drot_h1 as in afq_propagate_phaseless_jvp. With orbital rotation
 * (sampler.propagate_phaseless_ad, sampling.py:173-196, and its _nosr variant 221-254: the
 * trial re-optimised for h1 + lambda D by trial.optimize) also the trial's tangent
 * dtrial_up/dn [norb, n_s] (dn NULL for the RHF trial) and rot_chol's tangent
 * drot_chol_up/dn (layout of rot_chol_up/dn); all NULL for a fixed trial. The mean-field
 * shifts do not change (they follow wave_data["rdm1"], which the driver holds fixed). */
typedef struct afq_jvp_inputs {
  const double* dexp_h1_up;
  const double* dexp_h1_dn;
  const double* drot_h1_up;
  const double* drot_h1_dn;
  const double* dtrial_up;
  const double* dtrial_dn;
  const double* drot_chol_up;
  const double* drot_chol_dn;
} afq_jvp_inputs;

/* afq_propagate_phaseless_jvp with the tangent inputs in a struct, which adds the trial's
 * tangents of the orbital-rotation variants. The same workspace, flags and outputs. */
int afq_propagate_phaseless_jvp_ex(afq_ctx* ctx, afq_walker_state* state, const afq_jvp_inputs* in,
                                   void* tangent_workspace, size_t tangent_workspace_bytes,
                                   const double* fields, const double* zetas, int32_t n_prop_steps,
                                   int32_t n_ene_blocks, int32_t n_sr_blocks, int32_t flags,
                                   double* block_energy, double* block_weight, double* dblock_energy,
                                   double* dblock_weight, double* energy, double* denergy, void* stream);

/* ---- reverse-mode derivative of the block (differentiation pattern, FP64) ------------ */

/* Bytes of device workspace afq_propagate_phaseless_vjp needs for these block counts (the
 * recorded forward sweep grows with n_prop_steps * n_ene_blocks * n_sr_blocks). 0 on bad
 * sizes. */
size_t afq_vjp_workspace_size(const afq_dims* dims, int32_t n_prop_steps, int32_t n_ene_blocks,
                              int32_t n_sr_blocks);

/* afq_propagate_phaseless together with the gradient of its energy with respect to the
 * propagator's exp_h1 and the measurement intermediate rot_h1, the trial held fixed: the
 * reverse pass of the vjp that driver.py:217-229 takes of
 * sampler.propagate_phaseless_ad_norot (sampling.py:266-285; with AFQ_JVP_NO_SR in flags the
 * _nosr_norot variant, 287-317) with cotangent 1 on the energy. The caller maps the two
 * gradients to d energy / d h1 (the block's one-body density matrix estimate) through the
 * transposed Frechet derivative of expm and the trial's rotation. Outputs (device, float64,
 * overwritten): gexp_h1_up/dn [norb, norb] per walker slab (dn NULL for restricted walkers)
 * and grot_h1_up/dn with the layout of rot_h1_up/dn (dn NULL for the RHF trial). Values
 * (walkers, weights, overlaps, scalars, block_energy, block_weight, energy) are those of
 * afq_propagate_phaseless on the same draws. Clamped quantities (weights set to 0, local
 * energies replaced by e_estimate) pass no gradient, as jnp.where's transpose gives.
 * vjp_workspace: 256-B aligned device memory of afq_vjp_workspace_size(dims, ...) bytes; it
 * records the forward sweep (walkers, weights, overlaps and shifts before every step and
 * around every QR) and holds the backward sweep's cotangents. FP64 contexts only. */
int afq_propagate_phaseless_vjp(afq_ctx* ctx, afq_walker_state* state, void* vjp_workspace,
                                size_t vjp_workspace_bytes, const double* fields, const double* zetas,
                                int32_t n_prop_steps, int32_t n_ene_blocks, int32_t n_sr_blocks,
                                int32_t flags, double* block_energy, double* block_weight,
                                double* energy, double* gexp_h1_up, double* gexp_h1_dn,
                                double* grot_h1_up, double* grot_h1_dn, void* stream);

/* Outputs of afq_propagate_phaseless_vjp_ex (device float64, overwritten; NULL where not
 * wanted or not applicable): the gradients of afq_propagate_phaseless_vjp, and for the
 * orbital-rotation variant (sampler.propagate_phaseless_ad, the trial re-optimised for
 * h1 + lambda D) also d energy / d trial per spin of the trial (gtrial_up/dn [norb, n_s], dn
 * NULL for the RHF trial) and d energy / d rot_chol in the layout [nchol][ktot], ktot =
 * (n_up [+ n_dn for UHF]) * norb, each row the up block followed by the dn block. The caller
 * maps them to d energy / d h1 through the transposed tangents of trial.optimize. */
typedef struct afq_vjp_outputs {
  double* gexp_h1_up;
  double* gexp_h1_dn;
  double* grot_h1_up;
  double* grot_h1_dn;
  double* gtrial_up;
  double* gtrial_dn;
  double* grot_chol;
  /* Cholesky-vector gradients, all three or none (the 2-RDM variant,
   * sampler.propagate_phaseless_ad_1, sampling.py:198-229, rebuilds chol from a two-body
   * operator): d energy / d chol [nchol][norb^2] through the vhs contraction, d energy /
   * d mf_shifts [nchol] complex and d energy / d h0_prop (one complex). */
  double* gchol;
  double* gmf_shifts;
  double* gh0_prop;
} afq_vjp_outputs;

/* afq_propagate_phaseless_vjp with the outputs in a struct (the trial and rot_chol
 * gradients of the orbital-rotation variant added). */
int afq_propagate_phaseless_vjp_ex(afq_ctx* ctx, afq_walker_state* state, void* vjp_workspace,
                                   size_t vjp_workspace_bytes, const double* fields, const double* zetas,
                                   int32_t n_prop_steps, int32_t n_ene_blocks, int32_t n_sr_blocks,
                                   int32_t flags, double* block_energy, double* block_weight,
                                   double* energy, const afq_vjp_outputs* out, void* stream);

/* ---- correlated sampling (ad_afqmc/corr_sample/corr_sample.py) ---------------------- */

/* One correlated-sampling block of one system with the given fields (float64
 * [n_prop_steps, nw, nchol]): n_prop_steps phaseless steps, killed-walker count, QR,
 * overlaps, local energies clamped to e_estimate beyond sqrt(2/dt), block energy and weight,
 * pop_control_ene_shift <- 0.9 shift + 0.1 block energy. No stochastic reconfiguration.
 * local_energies (float64 [nw], may be NULL), block_energy and block_weight (one double each)
 * are device pointers. Replaces corr_sample.field_block_scan (corr_sample.py:514-555) with
 * the en_samples clamp (482-491). */
int afq_field_block(afq_ctx* ctx, afq_walker_state* state, const double* fields,
                    int32_t n_prop_steps, double* local_energies, double* block_energy,
                    double* block_weight, void* stream);

/* Weight-outlier removal of a correlated pair, then the step sums of cs_steps_scan:
 * z_i = |w_i - mean(w)| / std(w) (population std) for each system, and every walker whose
 * larger z exceeds z_thresh gets weight 0 in both systems; sums[0..3] = (sum e1 w1,
 * sum w1, sum e2 w2, sum w2) over the updated weights. Device pointers; weights updated in
 * place. Replaces corr_sample.corr_otler_rm (corr_sample.py:557-594) and the sums of
 * cs_steps_scan.cs_step (corr_sample.py:673-694). */
int afq_cs_outlier_removal(double* weights1, double* weights2, const double* local_energies1,
                           const double* local_energies2, int32_t n_walkers, double z_thresh,
                           double* sums, void* stream);

/* Standard normal draws (Philox4x32-10 + Box-Muller), float64 [n], counter-based:
 * element i depends only on (seed, offset + i). Stands in for jax.random.normal in
 * sampling.py:61-69. */
int afq_fill_normal(double* out, int64_t n, uint64_t seed, uint64_t offset, void* stream);

/* Uniform [0,1) draws, same generator. Stands in for jax.random.uniform in
 * propagation.py:236-237. */
int afq_fill_uniform(double* out, int64_t n, uint64_t seed, uint64_t offset, void* stream);

/* ---- allocation-free variant --------------------------------------------------------
 * No counterpart in the reference. For callers that cannot allocate device memory (code
 * running inside another runtime's memory arena, such as a JAX/XLA custom call that only
 * receives pre-allocated buffers, or a process whose device memory is reserved up front):
 * the force bias of afq_calc_force_bias for an RHF trial and restricted complex128 walkers,
 * in FP64, with no context, no workspace and no allocation. The Green's function it needs
 * as scratch lives in a 40 MiB static device array inside the library (held by every GPU
 * that loads the library until the process exits), so n_walkers * nocc * norb must not
 * exceed 2,621,440; larger sizes return a negative code with a message.
 * trial: [norb, nocc] float64; rot_chol: [nchol, nocc, norb] float64; walkers:
 * [n_walkers, norb, nocc] complex128; force_bias: [n_walkers, nchol] complex128 (out).
 * The first call on each device looks up the array's device address (make that first call
 * before any stream capture). All calls share the one array: calls that overlap on the GPU
 * (other streams, other host threads) race; serialise them. */
int afq_calc_force_bias_noalloc(int32_t norb, int32_t nocc, int32_t nchol, int32_t n_walkers,
                                const double* trial, const double* rot_chol, const void* walkers,
                                double* force_bias, void* stream);

/* ---- launch accounting ----------------------------------------------------------------
 * Diagnostics with no counterpart in the reference (which has no profiler hooks). Every
 * kernel launch is counted per kernel class; with timing enabled, each launch is also
 * bracketed by a CUDA-event pair recorded on its own stream. */

/* Reset counters; on != 0 also records event pairs around every launch. */
int afq_profile_enable(int on);
int afq_profile_reset(void);
/* Launches of class `cls` since the last reset and, when timing is on, their summed
 * device time in milliseconds (synchronises on the recorded events). */
int afq_profile_read(int cls, double* total_ms, int64_t* launches);
const char* afq_profile_class_name(int cls);
int afq_profile_num_classes(void);

#ifdef __cplusplus
}
#endif
#endif /* AFQMC_GB300_H */
