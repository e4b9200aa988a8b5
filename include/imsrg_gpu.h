/*
 * imsrg_gpu.h -- C ABI of the GB300 IMSRG(2) commutator engine.
 *
 * Drop-in boundary for the scalar-operator hot path of
 * n-parzuchowski/EOM-IMSRG_FULL (paths below are relative to im-SRG/).  Each
 * entry point names the Fortran routine it replaces.  A Fortran caller binds
 * these with ISO_C_BINDING interfaces (bind(C, name=...), integer(c_int),
 * value), in the style the reference already uses for zlib in gzipmod.f90:5-39.
 *
 * Conventions
 *  - Every function returns an int status: IMSRG_OK (0) or an IMSRG_ERR_*
 *    code.  Nothing aborts or exits the calling process.
 *  - Orbit arrays are 0-based C arrays of length norb holding the values of
 *    the reference's jbas%nn, %ll, %jj (= 2j), %itzp (= 2tz), %con (1 hole,
 *    0 particle), in the reference orbit order.
 *  - Matrices are Fortran column-major, exactly as the reference allocates
 *    them in allocate_blocks (basic_IMSRG.f90:477-641): per (2J,Tz,parity)
 *    block q = 3*2J + 2*(Tz+1) + parity + 1 the six arrays gam(1..6) =
 *    pppp (npp,npp), ppph (npp,nph), pphh (npp,nhh), phph (nph,nph),
 *    hhhh (nhh,nhh), phhh (nph,nhh), with rows/columns in the pair order of
 *    the block's qn lists.  One-body: fhh (A,A), fph (P,A), fpp (P,P).
 *  - The "flat" layout used by the *_flat calls is
 *        [E0 | fhh | fph | fpp | q=1..nblocks: gam(1..6)]
 *    with no padding (imsrg_basis_info_t::nfull doubles).
 *  - The "packed" layout is the reference's vectorize order
 *    (basic_IMSRG.f90:3794-3918, length neq), the format of its operator
 *    checkpoints.
 *  - All device work of one basis runs, in order, on that basis's CUDA
 *    stream.  Calls that return host values synchronise that stream.  A basis
 *    and its operators must be used from one host thread at a time.
 *  - The library keeps no global mutable state apart from these handles (the
 *    reference's v_elem/v_same COMMON cache, basic_IMSRG.f90:1282, is not
 *    mirrored).
 */
#ifndef IMSRG_GPU_H
#define IMSRG_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  IMSRG_OK = 0,
  IMSRG_ERR_INVALID = 1,        /* bad argument, shape or handle */
  IMSRG_ERR_CUDA = 2,           /* CUDA runtime error */
  IMSRG_ERR_OOM = 3,            /* device allocation failed */
  IMSRG_ERR_NOT_CONVERGED = 4,  /* BCH series clipped (IMSRG_MAGNUS.f90:232) */
  IMSRG_ERR_NONFINITE = 5,      /* NaN/Inf detected in a result */
  IMSRG_ERR_TIMEOUT = 6,        /* a bounded device wait gave up */
  IMSRG_ERR_MISMATCH = 7,       /* operators of different bases */
  IMSRG_ERR_NO_DEVICE = 8,      /* no usable CUDA device */
  IMSRG_ERR_TOO_LARGE = 9,      /* basis exceeds a fixed workspace limit */
  IMSRG_ERR_IO = 10             /* checkpoint file error */
};

/* Arithmetic of the dense two-body contractions (222_pp_hh ladders and the
 * particle-hole WCC product).  Everything else is always FP64. */
enum {
  IMSRG_PREC_FP64 = 0,   /* plain FP64 */
  IMSRG_PREC_OZAKI = 1   /* FP64 operands split into BF16 slices on tcgen05
                            tensor cores, exact FP32 slice products,
                            recombined in FP64 */
};

/* Generators of the flow (the reference's magnus_decouple takes one as an
 * external procedure, IMSRG_MAGNUS.f90:29, main_IMSRG.f90:216). */
enum {
  IMSRG_GEN_WHITE = 0,  /* build_gs_white (generators.f90:4-106) */
  IMSRG_GEN_ATAN = 1,   /* build_gs_atan  (generators.f90:162-266) */
  IMSRG_GEN_W2 = 2      /* build_gs_w2    (generators.f90:109-159) */
};

typedef struct imsrg_basis imsrg_basis_t;
typedef struct imsrg_op imsrg_op_t;

typedef struct {
  int norb, nholes, nparts;
  int nblocks;       /* (Jtotal_max + 1) * 6 */
  int jtotal_max;    /* maxval(jj) */
  int ccblocks;      /* (Jtotal_max + 1) * 4 */
  long nfull;        /* doubles in the flat layout */
  long neq;          /* doubles in the packed (vectorize) layout */
  long cc_total;     /* doubles of one cross-coupled operator (all CCX) */
  long wcc_total;    /* doubles of the WCC workspace */
} imsrg_basis_info_t;

/* --- basis (replaces read_sp_basis/find_holes + allocate_blocks +
 *     allocate_CCMAT + store_6j: basic_IMSRG.f90:152-400, 477-641,
 *     2183-2288; cross_coupled.f90:61-177) ---------------------------- */
int imsrg_gpu_basis_create(int norb, const int *nn, const int *ll, const int *jj, const int *itzp,
                           const int *con, imsrg_basis_t **out);
int imsrg_gpu_basis_destroy(imsrg_basis_t *b);
int imsrg_gpu_basis_info(const imsrg_basis_t *b, imsrg_basis_info_t *info);
/* npp/nph/nhh of block q (1-based), as op%mat(q)%npp etc. */
int imsrg_gpu_block_dims(const imsrg_basis_t *b, int q, int *npp, int *nph, int *nhh);
/* Blocks until all queued work of the basis has finished. */
int imsrg_gpu_synchronize(imsrg_basis_t *b);

/* --- operators (replaces allocate_blocks/duplicate_sq_op storage,
 *     basic_IMSRG.f90:2736-2918) ------------------------------------- */
int imsrg_gpu_op_create(imsrg_basis_t *b, int herm, imsrg_op_t **out);
int imsrg_gpu_op_destroy(imsrg_op_t *op);
int imsrg_gpu_op_set_herm(imsrg_op_t *op, int herm);
int imsrg_gpu_op_get_herm(const imsrg_op_t *op, int *herm);
/* Fortran sq_op arrays: gam[(q-1)*6 + (g-1)] points to op%mat(q)%gam(g)%X. */
int imsrg_gpu_op_upload(imsrg_op_t *op, double e0, const double *fhh, const double *fph, const double *fpp,
                        const double *const *gam);
int imsrg_gpu_op_download(const imsrg_op_t *op, double *e0, double *fhh, double *fph, double *fpp,
                          double *const *gam);
int imsrg_gpu_op_upload_flat(imsrg_op_t *op, const double *flat);
int imsrg_gpu_op_download_flat(const imsrg_op_t *op, double *flat);
/* vectorize / repackage (basic_IMSRG.f90:3794-3918) */
int imsrg_gpu_op_upload_packed(imsrg_op_t *op, const double *packed);
int imsrg_gpu_op_download_packed(const imsrg_op_t *op, double *packed);
/* Device address of the flat layout (nfull doubles), for callers that keep
 * their own device buffers in the same layout. */
int imsrg_gpu_op_device_ptr(imsrg_op_t *op, double **dptr);
/* Operator files of write_omega_checkpoint / read_omega_checkpoint and
 * write_twobody_operator (basic_IMSRG.f90:3069-3312): the vectorize vector
 * (neq doubles, native byte order) as an unformatted stream, no header.
 * load requires exactly neq doubles and keeps the operator's herm. */
int imsrg_gpu_op_save(const imsrg_op_t *op, const char *path);
int imsrg_gpu_op_load(imsrg_op_t *op, const char *path);
/* The reference's checkpoint file name: dir, the run prefix up to its 'hw'
 * field plus two characters, '_s', s in f6.3 left-adjusted (a '0' appended
 * below s = 10), '.bin' (basic_IMSRG.f90:3142-3160).  Host only. */
int imsrg_gpu_checkpoint_name(const char *dir, const char *prefix, double s, char *out, int outlen);
/* normal_order (basic_IMSRG.f90:2375-2506) in place: E0 and the one-body part
 * of H become those of H normal-ordered with respect to the reference state;
 * one-body elements of different (l,j,tz) are left as they are. */
int imsrg_gpu_normal_order(imsrg_op_t *H);

/* copy_sq_op (basic_IMSRG.f90:2942-2969): dst = src, herm included */
int imsrg_gpu_op_copy(const imsrg_op_t *src, imsrg_op_t *dst);
/* clear_sq_op (basic_IMSRG.f90:3537-3562) */
int imsrg_gpu_op_clear(imsrg_op_t *op);
/* add_sq_op (basic_IMSRG.f90:3450-3478): C = ax*A + bx*B (C may alias A/B) */
int imsrg_gpu_op_add(const imsrg_op_t *A, double ax, const imsrg_op_t *B, double bx, imsrg_op_t *C);
/* mat_frob_norm (basic_IMSRG.f90:3921-3952) */
int imsrg_gpu_op_norm(const imsrg_op_t *op, double *out);
/* mbpt2 (basic_IMSRG.f90:4030-4064) */
int imsrg_gpu_op_mbpt2(const imsrg_op_t *H, double *out);
/* E0 of the operator (a device read) */
int imsrg_gpu_op_get_e0(const imsrg_op_t *op, double *e0);

/* --- commutator engine -------------------------------------------------
 * [L,R] into RES, which is overwritten; RES herm becomes -herm(L)*herm(R)
 * (brute_force_testing.f90:509).  Replaces the sequence
 *   calculate_cross_coupled(L), calculate_cross_coupled(R),
 *   commutator_110 + commutator_220, commutator_111, commutator_121,
 *   commutator_122, commutator_222_pp_hh, commutator_221, commutator_222_ph
 * of IMSRG_MAGNUS.f90:207-219 (commutators.f90:10-925,
 * cross_coupled.f90:1190-1300).  with_e0 = 0 skips 110/220 and leaves
 * RES E0 unchanged, as MAGNUS_EXPAND does (IMSRG_MAGNUS.f90:676-685).
 * RES must not alias L or R. */
int imsrg_gpu_commutator(const imsrg_op_t *L, const imsrg_op_t *R, imsrg_op_t *RES, int precision, int with_e0);
/* The same commutator on host operands in the flat layout (nfull doubles
 * each; RES herm = -herm_L herm_R), for callers whose operators live in host
 * memory as the reference's sq_op arrays do: L and R are copied in, the
 * result copied back, and the call returns when RES is written.  The copies
 * overlap the commutator where its order allows (the digit images of L start
 * while R is in flight); from page-locked (pinned) buffers the whole sequence
 * replays as one CUDA graph.  RES must not overlap L or R. */
int imsrg_gpu_commutator_host(imsrg_basis_t *b, const double *L, int herm_L, const double *R, int herm_R,
                              double *RES, int precision, int with_e0);
/* The same on host operands in the packed (vectorize) layout of
 * basic_IMSRG.f90:3794-3918 (neq doubles each: only the independent
 * elements, ~57 % of the flat layout at emax = 6), the form the reference's
 * ODE solver and checkpoints hold operators in.  Page-locked arrays the
 * device can address (cudaHostAlloc, or cudaHostRegister with mapping) are
 * read by the device's unpack kernels and the result is written by its pack
 * kernel in place, over the host link, with no staging copies (R's
 * unpacking and its half of the work run beside L's); other arrays are
 * copied in, unpacked, packed and copied back.  Square arrays' lower
 * triangles come from herm x the upper ones (repackage).  RES must not
 * overlap L or R, and none of the three may be touched by the caller until
 * the call returns.  From page-locked buffers the sequence replays as one
 * CUDA graph. */
int imsrg_gpu_commutator_host_packed(imsrg_basis_t *b, const double *L, int herm_L, const double *R, int herm_R,
                                     double *RES, int precision, int with_e0);

/* build_gs_white (generators.f90:4-106): ETA (herm -1) from H.  ETA E0 is
 * left unchanged, as in the reference. */
int imsrg_gpu_build_gs_white(const imsrg_op_t *H, imsrg_op_t *ETA);
/* build_gs_atan (generators.f90:162-266): the White denominators with
 * eta = atan(2 N / D) * 0.5. */
int imsrg_gpu_build_gs_atan(const imsrg_op_t *H, imsrg_op_t *ETA);
/* build_gs_w2 (generators.f90:109-159): ETA1 = atan(H), H2 = [ETA1, H],
 * ETA2 = atanxx(H, H2) (denominators from H, numerators from H2,
 * :271-376), ETA = 1.5 ETA1 + 0.5 ETA2; the commutator in `precision`. */
int imsrg_gpu_build_gs_w2(const imsrg_op_t *H, imsrg_op_t *ETA, int precision);

/* dHds (IMSRG_ODE.f90:416-463): DH = [eta(HS), HS] with the generator
 * IMSRG_GEN_*, the derivative the reference hands its Shampine-Gordon solver
 * (the solver stays with the caller; DH in packed form via
 * imsrg_gpu_op_download_packed is its yp vector). */
int imsrg_gpu_dhds(const imsrg_op_t *HS, imsrg_op_t *DH, int generator, int precision);

/* decouple_hamiltonian (IMSRG_ODE.f90:9-178), one operator: integrates
 * dHS/ds = [eta(HS), HS] with the Shampine-Gordon Adams solver of
 * adams_ode.f90 (ODE/DE/STEP/INTRP, :33-1357; the reference passes relerr =
 * abserr = 1e-6 and ds = 0.1) in output steps of ds, continuing the
 * integration across steps, until |E_mbpt2| < 1e-6, or s >= s_max when
 * s_max > 0 (not in the reference), or max_steps steps (the reference's
 * 10000).  HS (herm +1) is advanced in place.  trace receives
 * (step, s, E0, E0 + E_mbpt2, |E_mbpt2|) per step, (max_steps + 1) x 5
 * doubles, like the reference's _0bflow.dat; *steps_out the steps taken,
 * *nfev the derivative evaluations.  relerr/abserr may be raised by the
 * solver as the reference's are (its IFLAG 3). */
int imsrg_gpu_ode_decouple(imsrg_op_t *HS, int generator, int precision, double ds, double s_max, int max_steps,
                           double relerr, double abserr, double *trace, int *steps_out, long *nfev);

/* --- Magnus flow ------------------------------------------------------- */
/* MAGNUS_EXPAND (IMSRG_MAGNUS.f90:622-693): DG in = eta, out = dOmega/ds.
 * *ncomm = commutators evaluated. */
int imsrg_gpu_magnus_expand(imsrg_op_t *DG, const imsrg_op_t *G, int precision, int *ncomm);
/* BCH_EXPAND (IMSRG_MAGNUS.f90:149-234): HS = exp(G) H exp(-G).
 * Returns IMSRG_ERR_NOT_CONVERGED where the reference STOPs ('clipping BCH'). */
int imsrg_gpu_bch_expand(imsrg_op_t *HS, const imsrg_op_t *G, const imsrg_op_t *H, int precision, int *ncomm);
/* transform_sq_op_BCH (IMSRG_MAGNUS.f90:131-146), scalar operators:
 * Op = exp(G) Op exp(-G) by BCH_EXPAND, in place. */
int imsrg_gpu_transform_bch(imsrg_op_t *Op, const imsrg_op_t *G, int precision, int *ncomm);
/* euler_step (IMSRG_MAGNUS.f90:756-766): G += ds*DG, *s += ds */
int imsrg_gpu_euler_step(imsrg_op_t *G, const imsrg_op_t *DG, double *s, double ds);
/* magnus_decouple (IMSRG_MAGNUS.f90:15-128) with build_gs_white and an added
 * stop at s >= s_max.  HS: in = normal-ordered H, out = H(s).  G: out =
 * Omega(s).  trace (optional, 5*(max_steps+1) doubles) receives the rows
 * (step, s, E0, E0 + mbpt2, |mbpt2|) of the reference's _0b_magnus_flow.dat.
 * *steps = Magnus steps taken, *ncomm = commutators evaluated. */
int imsrg_gpu_magnus_decouple(imsrg_op_t *HS, imsrg_op_t *G, double s_max, double ds, int max_steps, int precision,
                              double *trace, int *steps, int *ncomm);
/* The same flow with the generator IMSRG_GEN_* (imsrg_gpu_magnus_decouple
 * is generator IMSRG_GEN_WHITE). */
int imsrg_gpu_magnus_decouple_gen(imsrg_op_t *HS, imsrg_op_t *G, int generator, double s_max, double ds,
                                  int max_steps, int precision, double *trace, int *steps, int *ncomm);
/* The same flow with each Magnus step one CUDA graph launch: the Magnus and
 * BCH series run as device-side conditional loops, and the host reads back
 * only the step's scalars.  Results are bit-identical to
 * imsrg_gpu_magnus_decouple.  (No reference counterpart: the reference's
 * loop is the host-driven one.)  The graph is built on the first call for an
 * (HS, G, precision, ds) set and reused. */
int imsrg_gpu_magnus_decouple_graph(imsrg_op_t *HS, imsrg_op_t *G, double s_max, double ds, int max_steps,
                                    int precision, double *trace, int *steps, int *ncomm);
/* n independent flows advanced together: HS[i], G[i] on their own bases
 * (each instance needs its own workspace; a shared basis is rejected).
 * Every round launches one step graph per unfinished instance on its
 * basis's stream, so instances overlap on the device; each result equals its
 * unbatched flow bit for bit.  traces[i] (optional) as above; steps, ncomm and
 * status (optional) are n-element arrays.  Returns the first non-OK status. */
int imsrg_gpu_magnus_decouple_batch(int n, imsrg_op_t *const *HS, imsrg_op_t *const *G, double s_max, double ds,
                                    int max_steps, int precision, double *const *traces, int *steps, int *ncomm,
                                    int *status);
/* The reference's step-size and checkpoint-period rules of magnus_decouple
 * (IMSRG_MAGNUS.f90:45-51, 56-62), which the flow entry points leave to the
 * caller: ds = 0.5 for lawson_beta < 6, else 0.1; a checkpoint every chk = 4
 * steps at eMax = 14, every step above, every 24 below (eMax = max 2n+l of
 * the basis).  Either output may be NULL.  Host only. */
int imsrg_gpu_magnus_rules(const imsrg_basis_t *b, double lawson_beta, double *ds, int *chk);
/* magnus_decouple with the reference's Omega checkpoints
 * (IMSRG_MAGNUS.f90:56-110; write_omega_checkpoint and read_omega_checkpoint,
 * basic_IMSRG.f90:3132-3312).  With dir and prefix non-NULL:
 *  - at the start the newest checkpoint is looked for as the reference does
 *    (s = 95.5, 95.0, ... down to 1.5, file names of
 *    imsrg_gpu_checkpoint_name); when one is found the flow restarts from it:
 *    G = Omega(sx), HS = BCH_EXPAND(G, H) with H the HS passed in, the
 *    generator of HS, s = sx, step counter nint(sx/ds), and *s_restart = sx
 *    (else -1);
 *  - before the Magnus step of every step count divisible by chk (chk <= 0:
 *    the imsrg_gpu_magnus_rules value) Omega(s) is written to its file, except
 *    the first one due after a restart, and the file of s - 12 (eMax = 14:
 *    s - 4) is removed;
 *  - prefixes beginning with "testcase" write and read nothing.
 * The step is the host-driven one of imsrg_gpu_magnus_decouple_gen
 * (use_graph = 0; generator IMSRG_GEN_*) or the graph launch of
 * imsrg_gpu_magnus_decouple_graph (use_graph = 1; White generator only), so a
 * restarted flow takes the uninterrupted one's steps; H and Omega agree with
 * it to rounding (the file format keeps upper triangles and writes square
 * diagonals as herm x stored value, which flips the sign of the rounding
 * residue on the diagonals of the anti-Hermitian Omega).  trace rows
 * are indexed by the step counter (a restarted flow leaves the rows up to its
 * restart step untouched, as the reference appends to its flow file);
 * *steps is the final step counter, *ncomm the commutators of this call. */
int imsrg_gpu_magnus_decouple_checkpoint(imsrg_op_t *HS, imsrg_op_t *G, int generator, double s_max, double ds,
                                         int max_steps, int precision, int use_graph, const char *dir,
                                         const char *prefix, int chk, double *trace, int *steps, int *ncomm,
                                         double *s_restart);
/* Derivative of the flow along one direction of the input Hamiltonian
 * (forward mode; no reference counterpart).  dHS: in = dH(0) (for
 * H(c) = T + sum_k c_k V_k, the normal-ordered V_k gives dE0/dc_k), out =
 * dH(s).  dG: out = dOmega(s).  Every nested commutator T_n = [G, T_n-1] of
 * the Magnus and BCH series carries dT_n = [dG, T_n-1] + [G, dT_n-1]; the
 * White generator carries its tangent (d eta = (dN - eta dD)/D); term counts
 * and stops follow the undifferentiated flow, which runs alongside in HS, G
 * exactly as in imsrg_gpu_magnus_decouple.  dtrace (optional, as trace)
 * receives (step, s, dE0, 0, 0). */
int imsrg_gpu_magnus_decouple_tangent(imsrg_op_t *HS, imsrg_op_t *dHS, imsrg_op_t *G, imsrg_op_t *dG, double s_max,
                                      double ds, int max_steps, int precision, double *trace, double *dtrace,
                                      int *steps, int *ncomm);

/* --- reverse-mode derivatives (no reference counterpart: the reference has no
 *     derivative code; its checks are finite differences of the flow) ------
 * Adjoint of the two-body commutator: for a fixed X, the commutator RES =
 * [X, Y] of imsrg_gpu_commutator (the sequence of IMSRG_MAGNUS.f90:207-219)
 * is linear in Y, and
 *     Ybar = d <Cbar, [X, Y]> / dY      (<A, B> = sum over the flat layout)
 * is its transpose applied to Cbar, for Y of hermiticity herm_Y (Ybar herm
 * herm_Y, overwritten).  Every forward piece (Pandya transform, ladder and
 * WCC products, recoupling, 122/121/221/111 insertions, 110/220 energy) is
 * transposed on the forward's own gather lists; FP64.  with_e0 = 0 is the
 * commutator that leaves RES E0 alone (MAGNUS_EXPAND's), so Cbar E0 is
 * ignored.  The derivative with respect to X is -(the same call with X and Y
 * swapped), since [X, Y] = -[Y, X].  Scatters use FP64 atomics: results agree
 * run to run to rounding, not bit for bit. */
int imsrg_gpu_commutator_adjoint(const imsrg_op_t *X, const imsrg_op_t *Cbar, int herm_Y, int with_e0,
                                 imsrg_op_t *Ybar);
/* Adjoint of build_gs_white (generators.f90:4-106) at H: Hbar = (d eta / dH)^T
 * ETAbar (overwritten, herm of H).  FP64 atomics, as above. */
int imsrg_gpu_white_adjoint(const imsrg_op_t *H, const imsrg_op_t *ETAbar, imsrg_op_t *Hbar);
/* <A, B> over the flat layout (fixed summation order). */
int imsrg_gpu_op_dot(const imsrg_op_t *A, const imsrg_op_t *B, double *out);
/* The Magnus flow of imsrg_gpu_magnus_decouple (White generator; same
 * arguments, results and trace) followed by one backward sweep of its
 * adjoint: Hbar (may be NULL; herm +1) receives the gradient of the final E0
 * with respect to every element of the input HS (flat layout), and grad[j] =
 * <Hbar, dirs[j]> for j < ndir.  For H(c) = T + sum_k c_k V_k with HS =
 * normal_order(H(c)), dirs[k] = normal_order(V_k) gives grad[k] = dE0/dc_k
 * for every k from one sweep.  The forward keeps every Magnus and BCH term
 * in device memory (one operator each; about the flow's commutator count x
 * nfull doubles) and runs in `precision`; the backward sweep's transposed
 * commutators are FP64.  The series keep the forward flow's term counts. */
int imsrg_gpu_magnus_decouple_adjoint(imsrg_op_t *HS, imsrg_op_t *G, imsrg_op_t *Hbar, double s_max, double ds,
                                      int max_steps, int precision, int ndir, const imsrg_op_t *const *dirs,
                                      double *grad, double *trace, int *steps, int *ncomm);

/* The split-precision engine's CTA schedule (no reference counterpart): when
 * a basis first runs a split-precision commutator, the engine times its
 * persistent tensor-core kernel under *ncand candidate tile-cost models and
 * keeps the fastest (*choice); us[k] (up to max entries) receives each
 * candidate's time in microseconds.  IMSRG_ERR_INVALID before that first
 * use.  That first use allocates and synchronises, so it must not happen
 * inside a stream capture. */
int imsrg_gpu_split_schedule(imsrg_basis_t *b, int *choice, int *ncand, double *us, int max);
/* Pins that schedule to candidate model (0 <= model < ncand) without timing
 * (no reference counterpart): for runs whose event timings do not reflect
 * the kernel alone, such as under a profiler that serialises launches.  The
 * schedule never changes results.  Allocates and synchronises on first use. */
int imsrg_gpu_split_schedule_set(imsrg_basis_t *b, int model);
/* Digits per operand of IMSRG_PREC_OZAKI on this basis (no reference
 * counterpart): 6 (the default; 21 BF16 products per term, about 2^-42
 * K max|A| max|B| from the exact product), 5 (15 products, about 2^-35
 * K max|A| max|B|), 4 (10 products, about 2^-28 K max|A| max|B|), or the
 * FP64-class counts 7 and 8 (28 and 36 products, about 2^-49 and 2^-56
 * K max|A| max|B|, every digit level summed exactly, FP64 rounding of the
 * final sum).  Only before the basis' first split-precision call; later
 * it accepts the current count only (IMSRG_ERR_INVALID otherwise). */
int imsrg_gpu_split_digits_set(imsrg_basis_t *b, int digits);
/* Contraction chunking of IMSRG_PREC_OZAKI (no reference counterpart).  A
 * tile's digit products accumulate exactly in FP32 for at most 51 K steps of
 * 16 (steps x 16 x 5 x 2^12 < 2^24; 28 and 25 steps at seven and eight
 * digits, where every level stays exact); longer contractions (a term count
 * times K above 816, e.g. the pppp blocks from emax = 8 on) run in chunks,
 * each into its own accumulators, whose exact int64 level sums the epilogue
 * adds before converting once (at seven and eight digits each chunk's FP64
 * value).  steps > 0 caps the chunk at fewer steps (testing
 * and tuning; the result stays within the same error bound), 0 restores the
 * default.  Only before the basis' first split-precision call, like
 * imsrg_gpu_split_digits_set. */
int imsrg_gpu_split_chunk_set(imsrg_basis_t *b, int steps);

const char *imsrg_gpu_strerror(int status);
/* Number of library kernel launches issued so far on this basis. */
int imsrg_gpu_launch_count(const imsrg_basis_t *b, long *count);

/* --- streams and instrumentation (no reference counterpart) ------------ */
/* The cudaStream_t all work of the basis runs on.  set_stream makes the
 * library enqueue on a caller-owned stream instead (NULL restores its own). */
int imsrg_gpu_basis_get_stream(imsrg_basis_t *b, void **stream);
int imsrg_gpu_basis_set_stream(imsrg_basis_t *b, void *stream);
/* Kernel timing with CUDA events on the basis stream, per kernel class
 * IMSRG_KERNEL_*.  read returns the summed milliseconds and launch count
 * since the last reset (it synchronises the stream). */
enum {
  IMSRG_KERNEL_CC_FORWARD = 0,
  IMSRG_KERNEL_GEMM_FP64 = 1,
  IMSRG_KERNEL_ASSEMBLE_2BODY = 2,
  IMSRG_KERNEL_ASSEMBLE_1BODY = 3,
  IMSRG_KERNEL_OZAKI_SLICE = 4,
  IMSRG_KERNEL_OZAKI_MMA = 5,
  IMSRG_KERNEL_OZAKI_EPILOGUE = 6,
  IMSRG_KERNEL_OPS = 7,
  IMSRG_KERNEL_COUNT = 8
};
int imsrg_gpu_profile_enable(imsrg_basis_t *b, int on);
int imsrg_gpu_profile_read(imsrg_basis_t *b, int kernel, double *ms, long *launches);
int imsrg_gpu_profile_reset(imsrg_basis_t *b);

/* --- batches of independent commutators ------------------------------------
 * Many Hamiltonians at once (e.g. a scan over hbar*omega or coupling
 * constants): one commutator [L_i, R_i] per basis i, the split-precision
 * products of all bases in ONE persistent tensor-core launch (their tiles
 * scheduled longest first over the GPU together), the rest of each
 * commutator on that basis's own streams beside the others.  The reference
 * runs one commutator_* sequence per Hamiltonian (IMSRG_MAGNUS.f90:207-219).
 * imsrg_gpu_batch_create takes n distinct bases (each keeps its own
 * workspace; they must outlive the batch) and prepares the merged plan.
 * imsrg_gpu_batch_commutator computes RES_i = [L_i, R_i] for every i (each
 * operator of basis i; one herm_L and one herm_R for the whole batch;
 * RES_i herm = -herm_L herm_R) in either precision (FP64: the products of
 * all bases as one grouped FP64 launch), results identical to
 * imsrg_gpu_commutator, and
 * returns when all are done.  Each step is one cached CUDA graph per argument
 * set. */
typedef struct imsrg_batch imsrg_batch_t;
int imsrg_gpu_batch_create(int n, imsrg_basis_t *const *bases, imsrg_batch_t **out);
int imsrg_gpu_batch_commutator(imsrg_batch_t *batch, imsrg_op_t *const *L, imsrg_op_t *const *R,
                               imsrg_op_t *const *RES, int precision, int with_e0);
int imsrg_gpu_batch_destroy(imsrg_batch_t *batch);
/* magnus_decouple (IMSRG_MAGNUS.f90:15-128, White generator) of the batch's
 * n instances in lockstep: HS[i] (herm +1; in = normal-ordered H, out =
 * H(s)) and G[i] (out = Omega(s)) on the batch's basis i.  Each Magnus step is
 * ONE CUDA graph launch for all instances: the Magnus and BCH series loop on
 * the device while any instance's series runs; every series term computes
 * the split-precision products of all instances whose series still runs in
 * ONE persistent tensor-core launch (FP64: one grouped FP64 launch; the
 * others' tiles are skipped); instances whose series or flow has stopped
 * are skipped by conditional graph nodes.  Each instance's results, trace and
 * counts equal its unbatched imsrg_gpu_magnus_decouple_graph flow bit for
 * bit.  traces, steps, ncomm, status as in imsrg_gpu_magnus_decouple_batch.
 * The step graph is built on the first call for an (HS, G, precision, ds)
 * set and reused.  No reference counterpart (the reference runs one flow per
 * Hamiltonian). */
int imsrg_gpu_batch_magnus_decouple(imsrg_batch_t *batch, imsrg_op_t *const *HS, imsrg_op_t *const *G,
                                    double s_max, double ds, int max_steps, int precision, double *const *traces,
                                    int *steps, int *ncomm, int *status);

/* --- setup: interaction file, one-body HO part, Hartree-Fock ---------------
 * imsrg_gpu_read_interaction replaces read_interaction (interaction_IO.f90:
 * 8-107): the ASCII two-body file of VRenormalize (eight header lines, then
 * "Tz Par 2J a b c d V" per line, orbits 1-based in the basis order).  H is
 * cleared, then every element read is stored with the reference's pair
 * phases (normalised kets, hermitian input assumed) after the centre-of-mass
 * correction V += (beta (p1.p2 + (com_hw/hw)^2 r1.r2) - [htype == 1] p1.p2)
 * hw / mass (the r1.r2 and p1.p2 HO matrix elements of basic_IMSRG.f90:
 * 4310-4530).  H must have herm +1.  IMSRG_ERR_IO if the file cannot be read
 * or a line is malformed, IMSRG_ERR_INVALID for an orbit outside the basis. */
int imsrg_gpu_read_interaction(imsrg_op_t *H, const char *path, int htype, double hw, double com_hw,
                               double lawson_beta, int mass);
/* calculate_h0_harm_osc (basic_IMSRG.f90:2049-2147): sets fhh, fph and fpp of
 * H to the HO kinetic matrix of htype 1 (T - Tcm, Lawson-modified when
 * |lawson_beta| >= 1e-5), 2 (T + U_HO), 3 (T), 4 (T / mass) or 5 (the Hcm
 * one-body part); E0 and the two-body part are left as they are. */
int imsrg_gpu_h0_harm_osc(imsrg_op_t *H, int htype, double hw, double com_hw, double lawson_beta, int mass);
/* calc_HF (HF_mod.f90:14-106) without a three-body force: iterates the
 * Hartree-Fock equations of the (l, j, tz) blocks from the HO reference
 * until the summed eigenvalue change is below tol (the reference uses 1e-6),
 * at most max_iter times (IMSRG_ERR_NOT_CONVERGED beyond), then leaves H in
 * the normal-ordered HF basis: the one-body part is the Fock matrix in the HF
 * basis, the two-body part transformed, E0 = E_HF.  H holds T (one-body) and
 * V (two-body) on entry, not normal ordered (the reference's state after
 * read_interaction and calculate_h0_harm_osc).  coefs (may be NULL) receives
 * the HF coefficients D: norb x norb, column-major, D(a, i) the weight of HO
 * orbit a in HF orbit i (zero across blocks).  Density, Fock matrix,
 * diagonalisation and both transformations run on the GPU. */
int imsrg_gpu_hartree_fock(imsrg_op_t *H, double tol, int max_iter, double *e_hf, int *iterations, double *coefs);
/* observable_to_HF for a scalar operator (sqop_to_HF, HF_mod.f90:108-136):
 * the Hermitian operator Op (one- and two-body parts in the HO basis, not
 * normal ordered) is transformed with the HF coefficients coefs (norb x norb,
 * as imsrg_gpu_hartree_fock returns them) and normal ordered with respect to
 * the HF reference, in place. */
int imsrg_gpu_transform_to_hf(imsrg_op_t *Op, const double *coefs);

/* --- allocation-free commutator (no counterpart in the reference) --------
 * For callers that may not allocate device memory while they run: a host
 * program whose device memory is owned by another allocator or capped, code
 * running where a cudaMalloc/cudaFree (which can synchronise the whole
 * device) is not allowed, or a driver that reserves all memory up front.
 * Same result as imsrg_gpu_commutator(..., IMSRG_PREC_FP64, with_e0) on
 * caller-owned device buffers d_L, d_R, d_RES in the flat layout (nfull
 * doubles each; herm_L, herm_R = +1 or -1; RES herm is -herm_L*herm_R).  The
 * intermediates live in one fixed array of IMSRG_NOALLOC_SCRATCH_DOUBLES
 * doubles (8 MiB) that the library holds on every device that loads it, so
 * the call allocates nothing.  Bases whose intermediates (two flat
 * operators, the cross-coupled LCC and RCC, WCC, the 222_ph recoupling inputs
 * and the E0 partials) do not fit are rejected with IMSRG_ERR_TOO_LARGE
 * (emax <= 4 fits; emax = 6 does not).
 *  - The basis must have been created beforehand (creating it allocates the
 *    device tables once) and its device must be current.
 *  - The first call on each device is its set-up: it looks up the array's
 *    device address and loads the device code of the kernels this call
 *    launches (with CUDA's lazy module loading that would otherwise happen at
 *    their first launch, and loading can allocate and synchronise).  Make that
 *    first call before any stream capture and before the part of the program
 *    that must not allocate; later calls allocate nothing.
 *  - d_RES must not share any element with d_L or d_R (IMSRG_ERR_INVALID).
 *  - Work is enqueued on `stream` (NULL: the basis stream).  All calls share
 *    the one array, so calls that overlap on the GPU race; serialise them.
 *    The array keeps the last call's contents; every element a call reads is
 *    written earlier in the same call, so nothing needs clearing. */
#define IMSRG_NOALLOC_SCRATCH_DOUBLES 1048576
int imsrg_gpu_commutator_noalloc(imsrg_basis_t *b, const double *d_L, int herm_L, const double *d_R, int herm_R,
                                 double *d_RES, int with_e0, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* IMSRG_GPU_H */
