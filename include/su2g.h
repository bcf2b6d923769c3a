/*
 * su2g: GB300-native (sm_103a) SU(2) block-sparse DMRG hot path, C ABI.
 *
 * This header is the drop-in boundary between an SU2DMRG-style host engine and
 * the GPU library libsu2g.so.  Every entry point takes plain pointers and sizes
 * and returns an int status (SU2G_OK = 0); on failure su2g_last_error() gives
 * a one-line reason for the calling thread.  Nothing here calls exit().
 *
 * Block tensors (tensor_su2, tensor_su2.hpp:6-124) cross the boundary in the
 * reference's own checkpoint layout (dmrg_su2_omp.cpp:864-941):
 *   desc  int[]  = [nbond, locspin, {dir, n, angm[n], dim[n]} per leg]
 *                  angm = 2j of each sector in ascending order (su2bond),
 *                  dim  = multiplet count of the sector;
 *   flag  int[nten] = 1 where the block is stored, in mixed-radix block order
 *                  with leg 0 fastest (su2struct.cpp:243-261);
 *   data  double[] = the stored blocks back to back in block order, each a
 *                  column-major array of its multiplet dims (leg 0 fastest).
 * Only the reduced (multiplet) blocks travel; the Clebsch-Gordan part of each
 * block is the canonical one the reference engine uses (the singlet for 2-leg
 * vectors, make_cgc(j0,j1,j2) for 3-leg operators, the identity for 2-leg
 * scalar operators), so it is implied by the sector labels.
 *
 * "device" pointers are CUDA device addresses on the current device; "stream"
 * is a cudaStream_t passed as void* (NULL = legacy default stream).
 */
#ifndef SU2G_H
#define SU2G_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SU2G_OK 0
#define SU2G_EINVAL 1      /* inconsistent structures or arguments */
#define SU2G_ENOMEM 2      /* device allocation refused */
#define SU2G_ECUDA 3       /* a CUDA runtime call failed */
#define SU2G_ETIMEOUT 4    /* a bounded device wait gave up */
#define SU2G_EUNSUPPORTED 5
#define SU2G_EIO 6          /* a checkpoint file is missing, unreadable or malformed */

#define SU2G_MODE_F64 0             /* plain FP64 contractions (FP64 tensor-core MMA) */
#define SU2G_MODE_SPLIT_BF16 1      /* FP64 emulated with 7 BF16 digit slices on the tcgen05 tensor cores */
#define SU2G_MODE_SPLIT_BF16_FAST 2 /* the same with 6 slices: fewer products, about 2^-40 relative error */

typedef struct su2g_heff_plan su2g_heff_plan;

/* A block tensor: structure + presence flags (host) and packed data (device). */
typedef struct {
  const int* desc;
  const int* flag;
  const double* data;
} su2g_tensor;

/* One two-sided term  coef * op1 (x) op2  of the effective Hamiltonian. */
typedef struct {
  su2g_tensor op1; /* 3 legs: (left-in, operator spin, left-out)   */
  su2g_tensor op2; /* 3 legs: (right-in, operator spin, right-out) */
  double coef;
} su2g_term;

/* ---------------------------------------------------------------- meta -- */
/* Library version (major*10000 + minor*100 + patch). */
int su2g_version(void);
/* One-line reason for the last failure on this thread. */
const char* su2g_last_error(void);

/* Number of blocks of a structure (su2struct::get_nten, su2struct.hpp:27). */
int su2g_struct_nten(const int* desc);
/* legal[i] = 1 for every block that passes the reference's legality test
 * (su2struct::get_tensor_argument / check_angularmoments, su2struct.cpp:264-332).
 * Returns nten, or -1 for a malformed desc. */
int su2g_struct_legal(const int* desc, int* legal);
/* offsets[i] (doubles) of every stored block in the packed layout, -1 where
 * flag[i] == 0; returns the packed length, -1 for a malformed desc. */
int64_t su2g_layout(const int* desc, const int* flag, int64_t* offsets);
/* su2bond::fuse (su2bond.cpp:155-210): sectors of b1 (x) b2, ascending, 2j
 * capped at 38.  aout/dout need room for 64 sectors. */
int su2g_bond_fuse(int n1, const int* a1, const int* d1, int n2, const int* a2, const int* d2, int* nout,
                   int* aout, int* dout);
/* tensor::make_cgc (tensor.cpp:1353-1407), column-major (j1+1)(j2+1)(j3+1). */
int su2g_make_cgc(int j1, int j2, int j3, double* out);
/* fac_hamilt_vec[i][j][k] of dmrg_su2.cpp:759-766 at out[(i*m+j)*m+k]. */
int su2g_fac_hamilt_vec(int max_angm, double* out);
/* fac_operator_transformation_left (side 0) / _rght (side 1)[j][m][l][i][k][p]
 * of dmrg_su2.cpp:857-890 (0 where the reference leaves the entry unset). */
int su2g_fac_operator_transformation(int side, int j, int m, int l, int i, int k, int p, double* out);

/* -------------------------------------------------------------- H_eff -- */
/* Builds the device work list of one effective Hamiltonian
 *   y = hl_coef*H_L^T psi + hr_coef*psi H_R + sum_t coef_t (op1_t, op2_t) psi
 * for a two-site step.  Replaces the per-call term loop of
 * dmrg_su2::hamiltonian_vector_multiplication_idmrg (dmrg_su2.cpp:543-664) and
 * the block loops of tensor_su2::hamiltonian_vector_multiplication
 * (tensor_su2_dmrg_src.cpp:893-1041) and tensor_su2::contract for the spin-0
 * terms (tensor_su2.cpp:1255-1345, called at dmrg_su2.cpp:563-570).
 * psi_desc/psi_flag describe psi and y (2 legs, locspin 0).  hl/hr may be
 * NULL.  Operator data pointers are captured and must stay valid until the plan
 * is destroyed; their contents must be complete when the plan is created (in
 * split mode the operators are split into digit slices here, on a stream of
 * the library's own: synchronise the stream that wrote them first).
 * Allocates the work list and its scratch on the device. */
int su2g_heff_plan_create(const int* psi_desc, const int* psi_flag, int nterms, const su2g_term* terms,
                          const su2g_tensor* hl, double hl_coef, const su2g_tensor* hr, double hr_coef, int mode,
                          su2g_heff_plan** plan);
/* Host-only dry run of su2g_heff_plan_create: builds the work lists of the
 * given mode and checks every element access their kernels would make against
 * the extent of the block it reads or writes, without touching a GPU.  Same
 * arguments; outputs the algorithmic FLOPs of one application and the device
 * bytes the plan would hold beyond its work lists. */
int su2g_heff_plan_validate(const int* psi_desc, const int* psi_flag, int nterms, const su2g_term* terms,
                            const su2g_tensor* hl, double hl_coef, const su2g_tensor* hr, double hr_coef, int mode,
                            double* flops, int64_t* scratch_bytes);
/* Host-only digest of every field of the work lists su2g_heff_plan_create
 * would build for `mode` (they fix every sum's order: equal digests, equal
 * results bit for bit).  Absolute operand addresses enter it: pass the same
 * data pointers to compare two builds.  No counterpart in the reference; it
 * pins the planner in tests. */
int su2g_heff_plan_digest(const int* psi_desc, const int* psi_flag, int nterms, const su2g_term* terms,
                          const su2g_tensor* hl, double hl_coef, const su2g_tensor* hr, double hr_coef, int mode,
                          uint64_t* digest);
/* Reads and clears the plan's device error word (the split-precision kernels
 * record a bounded wait that gave up there).  SU2G_ETIMEOUT if one did. */
int su2g_heff_plan_status(su2g_heff_plan* plan, int* code);
/* Tile shapes of the FP64 engine by block-size class (the autotuner of
 * su2dmrg_gb300.autotune fills it from measurements; no counterpart in the
 * reference, whose per-block loop tensor_su2_dmrg_src.cpp:977-1006 calls one
 * DGEMM per block).  Buckets: M <= m_edges[i] (i < nm), N <= n_edges[j], the
 * last bucket of each open-ended; cls[i * nn + j] in 0..3 = tiles of 64 x 64,
 * 64 x 32, 32 x 64, 32 x 32.  Plans built afterwards use it; without a table
 * every block uses 64 x 64. */
int su2g_f64_tile_table(const int* m_edges, int nm, const int* n_edges, int nn, const int* cls);
/* The autotuner's measurement: nblocks independent M x N x K block products
 * in tiles of class cls, one launch, repeated reps times; *ms = device
 * milliseconds per launch. */
int su2g_f64_tile_bench(int M, int N, int K, int nblocks, int cls, int reps, double* ms, void* stream);
/* Test hook, no counterpart in the reference: stores a nonzero `code` in the
 * plan's error word from the host, as a device wait that gave up would, so a
 * test can check on the CPU side, without any device fault, that every later
 * result of the plan (su2g_lanczos on each of its exits) is refused with
 * SU2G_ETIMEOUT. */
int su2g_heff_plan_mark_failed(su2g_heff_plan* plan, int code);
/* flops: algorithmic FLOPs of one application; psi_len: packed length of psi
 * and y (doubles); scratch_bytes: device scratch held by the plan; ntiles:
 * output tiles of the two launch phases. */
int su2g_heff_plan_info(const su2g_heff_plan* plan, double* flops, int64_t* psi_len, int64_t* scratch_bytes,
                        int* ntiles);
/* Number of this library's kernels one su2g_heff_apply launches (memsets and
 * copies not counted). */
int su2g_heff_plan_launches(const su2g_heff_plan* plan, int* n);
/* y = H_eff psi (device pointers, psi_len doubles each, no aliasing). */
int su2g_heff_apply(su2g_heff_plan* plan, const double* psi, double* y, void* stream);
/* su2g_heff_apply with a CUDA event between its launches; waits for the
 * result and writes the duration (ms) of each launch to ms[0..*nlaunch):
 * FP64 mode: phase 1, phase 2; split modes: pack psi, phase 1, pack the
 * intermediates, phase 2, sum of the split phase-2 tiles. */
int su2g_heff_apply_profile(su2g_heff_plan* plan, const double* psi, double* y, void* stream, double* ms,
                            int* nlaunch);
int su2g_heff_plan_destroy(su2g_heff_plan* plan);
/* Adds the excited-state penalty of hamiltonian_vector_multiplication_idmrg
 * (dmrg_su2.cpp:611-622): every later application also does
 *   y -= weight * (o . psi) * o
 * with o a device vector in psi's layout (the reference's overlapvec[j]) that
 * must stay valid, and weight its gs_enr[j].  The dot product stays on the
 * device (deterministic reduction). */
int su2g_heff_plan_add_projector(su2g_heff_plan* plan, const double* o, double weight);

/* Linear combination out = sum_i coef[i] * ops[i] of operators of one
 * structure (the summed partner sum_k coup * opr[ir][k] that
 * hamiltonian_vector_multiplication_idmrg rebuilds on every call,
 * dmrg_su2.cpp:588-600, formed once per step instead; or hh[i] += ...).  The
 * output holds the union of the operands' blocks (layout from
 * su2g_operator_combine_layout: flags of that union, packed length); each
 * element is summed in operand order.  Blocks until done. */
int su2g_operator_combine_layout(int n, const su2g_tensor* ops, int* out_flag, int out_flag_cap, int64_t* out_len);
int su2g_operator_combine(int n, const su2g_tensor* ops, const double* coef, double* out, void* stream);

/* One-shot form of tensor_su2::hamiltonian_vector_multiplication(vec, op1, op2)
 * (tensor_su2_dmrg_src.cpp:893-1041): y = (op1, op2) vec with the recoupling
 * factors of fac_hamilt_vec.  y (device) uses vec's layout: op1's last leg must
 * equal vec's leg 0 and op2's last leg vec's leg 1, so the result can be added
 * to vec-shaped accumulators as the reference does (dmrg_su2.cpp:606-608). */
int su2g_hamiltonian_vector_multiplication(const int* vec_desc, const int* vec_flag, const double* vec,
                                           su2g_tensor op1, su2g_tensor op2, double* y, void* stream);

/* ------------------------------------------ several plans, shared launches */
/* Independent solves that share the GPU (a serving loop) reach their Lanczos
 * solves at the same time.  A batch applies several H_eff plans (one
 * precision mode) in shared launches: their work lists are concatenated and
 * their tiles dealt together over the persistent grid, so one application of
 * all of them costs the launches of one plan.  Each plan's result is
 * bit-identical to its own su2g_heff_apply.  No counterpart in the reference,
 * whose solves are separate processes; per plan this is
 * dmrg_su2::hamiltonian_vector_multiplication_idmrg (dmrg_su2.cpp:543-664).
 * The plans must outlive the batch and must not change (no new projectors)
 * while it exists. */
typedef struct su2g_heff_batch su2g_heff_batch;
int su2g_heff_batch_create(su2g_heff_plan* const* plans, int n, su2g_heff_batch** batch);
int su2g_heff_batch_destroy(su2g_heff_batch* batch);
/* total_len: sum of the plans' psi lengths; plan i's vector lies at the sum
 * of the lengths of plans 0..i-1 in the batch vectors */
int su2g_heff_batch_info(const su2g_heff_batch* batch, int64_t* total_len, int* nplans);
/* y = H x for every plan on its slice of the batch vectors x and y (device,
 * total_len doubles each); asynchronous on `stream` */
int su2g_heff_batch_apply(su2g_heff_batch* batch, const double* x, double* y, void* stream);
/* reads and clears the batch's error word (SU2G_ETIMEOUT: a bounded wait of a
 * shared split-GEMM launch gave up; every plan's result is then suspect) */
int su2g_heff_batch_status(su2g_heff_batch* batch);
/* lanczos_su2::lanczos1 (lanczos_su2.cpp:125-195) for every plan of the
 * batch in lockstep: psi[i] (device, plan i's layout) is the start vector and
 * receives the eigenvector; energy[i] and nmatvec[i] as su2g_lanczos returns
 * them, bit for bit (the same kernels in the same order per plan, each plan's
 * exits decided as there); the matvecs of all solves at a step share one set
 * of launches.  Blocks until done; SU2G_ETIMEOUT refuses every result. */
int su2g_heff_batch_lanczos(su2g_heff_batch* batch, double* const* psi, int mlanc, double* energy, int* nmatvec,
                            void* stream);

/* Allocation-free form of su2g_hamiltonian_vector_multiplication, for callers
 * that may not allocate device memory when they apply a term: engines that
 * reserve their whole HBM budget up front, per-term calls from many host
 * threads where cudaMalloc/cudaFree would synchronise the device, code running
 * inside another library's callbacks.  This entry point has no counterpart in
 * the reference.  Its intermediate blocks and work list live in fixed
 * file-scope device arrays (SU2G_NOALLOC_* below, about 40 MiB), held by every
 * GPU that loads libsu2g.so until the process exits; terms that need more are
 * refused with SU2G_EINVAL.  The first call on a device looks up the arrays'
 * device addresses (cudaGetSymbolAddress).  The call cannot be captured into
 * a CUDA graph (it copies its work list from host memory it frees on
 * return): on a capturing stream it returns SU2G_EUNSUPPORTED.  Calls share
 * the arrays.  Calls from several host threads on the
 * same stream are safe: each call queues its copies and launches under a
 * per-device lock, so stream order keeps them apart.  Calls on different
 * streams race on the arrays and must be serialised by the caller.  Same
 * arguments and result as su2g_hamiltonian_vector_multiplication,
 * asynchronous on `stream`. */
#define SU2G_NOALLOC_SCRATCH_DOUBLES 4194304 /* intermediate blocks: 32 MiB */
#define SU2G_NOALLOC_MAX_TILES 65536
#define SU2G_NOALLOC_MAX_SEGS 65536
int su2g_hamiltonian_vector_multiplication_noalloc(const int* vec_desc, const int* vec_flag, const double* vec,
                                                   su2g_tensor op1, su2g_tensor op2, double* y, void* stream);

/* -------------------------------------------------- environment updates -- */
/* tensor_su2::operator_transformation(uu, vv, op, flag)
 * (tensor_su2_dmrg_src.cpp:221-402): carries each operator op_t of the last
 * environment (3 legs: bond, operator spin, bond) through the MPS tensors uu
 * and vv (3 legs; leg `flag` attaches to the operator, the other of legs 0/1
 * is the spin-1/2 physical leg, leg 2 the new bond) into a new operator on
 * the new bond, with the fac_operator_transformation_{left,rght} factors.
 * Called for a batch: op[t] -> out[t] (device), all sharing uu and vv, in one
 * device pass.  Each out[t] must have the layout reported by
 * su2g_operator_transformation_layout for op[t]: structure (uu leg 2, op
 * leg 1, vv leg 2 inverted) with exactly the blocks some product reaches, as
 * the reference creates them.  mode: SU2G_MODE_* as for H_eff.  Blocks until
 * done. */
int su2g_operator_transformation_layout(su2g_tensor uu, su2g_tensor vv, int flag, su2g_tensor op, int* out_desc,
                                        int out_desc_cap, int* out_flag, int out_flag_cap, int64_t* out_len);
int su2g_operator_transformation(su2g_tensor uu, su2g_tensor vv, int flag, int nops, const su2g_tensor* ops,
                                 double* const* outs, int mode, void* stream);
/* tensor_su2::overlap_transformation(uu, vv, hh, flag)
 * (tensor_su2_dmrg_src.cpp:531-688): the same for 2-leg scalar operators (the
 * block Hamiltonian), output structure (uu leg 2, vv leg 2 inverted). */
int su2g_overlap_transformation_layout(su2g_tensor uu, su2g_tensor vv, int flag, su2g_tensor hh, int* out_desc,
                                       int out_desc_cap, int* out_flag, int out_flag_cap, int64_t* out_len);
int su2g_overlap_transformation(su2g_tensor uu, su2g_tensor vv, int flag, int nops, const su2g_tensor* hhs,
                                double* const* outs, int mode, void* stream);

/* The rest of a site update (dmrg_su2::prepare_site_operator_from_{left,right},
 * dmrg_su2_omp.cpp:319-825) as one batch over the MPS tensors uu, vv:
 *   SU2G_ENV_OVERLAP     overlap_transformation(uu, vv, x, flag)      x: 2-leg scalar operator
 *   SU2G_ENV_TRANSFORM   operator_transformation(uu, vv, x, flag)     x: 3-leg operator
 *   SU2G_ENV_INITIAL     operator_initial(uu, vv, site1, flag), or with x (2-leg) as endt
 *                        operator_initial(uu, vv, site1, x, flag)      (tensor_su2_dmrg_src.cpp:27-218)
 *   SU2G_ENV_PAIRUP      operator_pairup(uu, vv, x, site1, flag)      (tensor_su2_dmrg_src.cpp:691-890)
 *   SU2G_ENV_PERMUTATION permutation(uu, vv, x, site1, site2, flag)   (tensor_su2_hamiltonian.cpp:871-1108)
 * x lives on the device; site1/site2 are the engine's site operators (sigma,
 * qterm, ...) with their data on the HOST.  Each job adds coef times its
 * result to outs[slot]; jobs naming one slot must produce the same structure
 * and are summed (the reference's hh[i] = overlap + sum of pairups).  The
 * layout of outs[slot] is what su2g_env_layout reports: the union of the
 * blocks the slot's jobs reach, as the reference creates them.  Physical legs
 * of uu, vv must have multiplicity 1; operator_initial needs single-element
 * site blocks; permutation needs an operator spin of multiplicity 1.  Blocks
 * until done. */
#define SU2G_ENV_OVERLAP 0
#define SU2G_ENV_TRANSFORM 1
#define SU2G_ENV_INITIAL 2
#define SU2G_ENV_PAIRUP 3
#define SU2G_ENV_PERMUTATION 4
typedef struct {
  int kind;          /* SU2G_ENV_* */
  int slot;          /* output index */
  double coef;       /* scale of this job's contribution */
  su2g_tensor x;     /* environment operator (device); desc NULL: none */
  su2g_tensor site1; /* site operator (host data) */
  su2g_tensor site2; /* second site operator of a permutation (host data) */
} su2g_env_job;
int su2g_env_layout(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int slot,
                    int* out_desc, int out_desc_cap, int* out_flag, int out_flag_cap, int64_t* out_len);
int su2g_env_run(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int nslots,
                 double* const* outs, int mode, void* stream);
/* Host-only dry run of su2g_env_run: builds and bounds-checks the work list
 * for `mode` (no device work, no allocation) and reports the algorithmic
 * flops and the device scratch it needs. */
int su2g_env_validate(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int nslots,
                      int mode, double* flops, int64_t* scratch_bytes);
/* Host-only digest of the work lists su2g_env_run would build (as
 * su2g_heff_plan_digest; the output addresses enter it too). */
int su2g_env_digest(su2g_tensor uu, su2g_tensor vv, int flag, int njobs, const su2g_env_job* jobs, int nslots,
                    double* const* outs, int mode, uint64_t* digest);

/* Recoupling factors of the site updates, computed on first use from the
 * Clebsch-Gordan contractions the reference tabulates (dmrg_su2.cpp:776-1019):
 *   table 0  fac_operator_onsite_{left,rght}[a][b][c][d][e]   (e = p0 + 3 p1)
 *   table 1  fac_operator_pairup_{left,rght}[a][b][c][d][e]   (e = p0 + 3 p1)
 *   table 2  fac_permutation_{left,rght}[a][b][c][d][e]       (e < 18, spin-1/2 sites)
 * side 0 = left, 1 = right; 0 where the reference leaves the entry unset. */
int su2g_fac_table(int table, int side, int a, int b, int c, int d, int e, double* out);

/* ---------------------------------------------------------- truncation -- */
/* vec.svd(tu, p1, tv, p2, dout, wout) (tensor_su2.cpp:1619-1758 with the
 * per-sector tensor::svd of tensor.cpp:1472-1700): splits the two-leg wave
 * function psi (device; legs = the fused legs 0, 1 of tu and of tv) back into
 * two MPS tensors, keeping the max_dcut largest multiplets over all spin
 * sectors (the reference's global max_dcut, passed here).  Per sector: Gram
 * matrix of the smaller side, FP64 eigendecomposition with the reference's
 * refinement of the small-eigenvalue subspace, values above 1e-100 of the
 * largest kept, columns scaled by s^p1 (U) and s^p2 (V); the global choice
 * uses the reference's Shell sort (sort2.f dsort2), so ties go the same way.
 *   tu_desc, tv_desc  3-leg descs of the current tu / tv: legs 0, 1 are used
 *   bond              out: the new bond [n, 2j[n], dim[n]] (direction -1),
 *                     bond_cap >= 1 + 2 * (sectors of psi leg 0)
 *   wout, dout        out: singular values, kept (per sector, ascending) then
 *                     discarded, as the reference writes them; *dout = count
 *   tu, tv            out (device, may be NULL): the new MPS tensors, layout
 *                     of [3, 0, tu leg 0, tu leg 1, (-1, bond)] (resp. tv)
 *                     with every legal block present (su2g_layout with a NULL
 *                     flag array); at most tu_cap / tv_cap doubles
 * The sectors run concurrently (one stream, handle pair and host thread
 * each, kept per device across calls); calls from several host threads take
 * turns.  Blocks until done. */
int su2g_svd(const int* psi_desc, const int* psi_flag, const double* psi, const int* tu_desc, double p1,
             const int* tv_desc, double p2, int max_dcut, int* bond, int bond_cap, double* wout, int wout_cap,
             int* dout, double* tu, int64_t tu_cap, double* tv, int64_t tv_cap, void* stream);

/* ------------------------------------------------------ between steps -- */
/* wavefunc_transformation(i, flag) (dmrg_su2_omp.cpp:1864-1876) on one MPS
 * tensor: tensor_su2::right2left_vectran (flag 0, legs (0,1,2) -> (2,0,1))
 * or left2right_vectran (flag 1, -> (1,2,0)) (tensor_su2.cpp:749-837).  Every
 * stored block moves to its rotated place with its legs rotated, numbers
 * unchanged (the canonical CG of the rotated spins, no factor); directions
 * become (+1, +1, -1).  out (device) has the layout su2g_vectran_layout
 * reports and the same length as u; out == u.data rotates in place, as the
 * reference does.  Apply it to uu[i] and to each orth[j][i].  Blocks until
 * done. */
int su2g_vectran_layout(su2g_tensor u, int flag, int* out_desc, int out_desc_cap, int* out_flag, int out_flag_cap,
                        int64_t* out_len);
int su2g_vectran(su2g_tensor u, int flag, double* out, void* stream);

/* tensor_su2::fuse(b1, b2) (tensor_su2.cpp:839-909), the MPS tensor the
 * warm-up starts each new site with (do_idmrg, dmrg_su2_omp.cpp:30-66): legs
 * (b1, b2, fuse(b1, b2) of direction -b1), every legal block present, each
 * block the rows of an identity placed where tensor_su2::fuse places them.
 * bonds_desc = a 2-leg desc holding b1 and b2 (locspin ignored); out (device)
 * has the layout su2g_fuse_tensor_layout reports. */
int su2g_fuse_tensor_layout(const int* bonds_desc, int* out_desc, int out_desc_cap, int* out_flag, int out_flag_cap,
                            int64_t* out_len);
int su2g_fuse_tensor(const int* bonds_desc, double* out, void* stream);
/* The warm-up's two-site start vector (prepare_input_vector_initial +
 * initialize_input_vector + normalize_vector, dmrg_su2_omp.cpp:196-216,
 * 79-80): the structure of su2g_prepare_input_vector's vector with every
 * element 1/sqrt(N), N its length. */
int su2g_initial_vector(su2g_tensor ul, su2g_tensor ur, double* out, void* stream);
/* The seeded random start vector: tensor_su2::random_initialize_tensor
 * (tensor_su2.cpp:2375-2393) followed by normalize_vector, in place of
 * initialize_input_vector at dmrg_su2_omp.cpp:79 (the -seed option added on
 * both sides).  out[k] = ran()*2 - 1 for k = 0..n-1 (the packed order of any
 * tensor's stored blocks), ran() the generator of ran.f90:2-16 continuing
 * from *state (initran: *state = seed), then out is divided by its norm
 * twice.  *state is advanced by n steps on return.  Blocks until done. */
int su2g_random_vector(int64_t* state, double* out, int64_t n, void* stream);

/* dmrg_su2::prepare_input_vector(il, ir, vec) (dmrg_su2_omp.cpp:229-254):
 * the initial two-site vector of a step from ul = uu[il] and ur = uu[ir]
 * (device data; legs 0 and 1 of each of one direction, leg 2 the same bond
 * in both).  vec has two legs, fuse(ul legs 0, 1) and fuse(ur legs 0, 1)
 * (su2bond::fuse) with the directions of ul leg 0 and ur leg 0, and every
 * block of equal spins (tensor_su2::makeup_input_vector,
 * tensor_su2.cpp:2334-2350): block (c, c) = U_L,c U_R,c^T, U the rows of an
 * MPS tensor's centre-spin-c blocks stacked in the order tensor_su2::fuse
 * places them, zero where no stored block reaches.  The same call gives the
 * excited-state vectors overlapvec[j] from ovlp[j][il], ovlp[j][ir].  mode:
 * SU2G_MODE_* for the block products.  out (device) has the layout
 * su2g_input_vector_layout reports.  Blocks until done. */
int su2g_input_vector_layout(su2g_tensor ul, su2g_tensor ur, int* out_desc, int out_desc_cap, int* out_flag,
                             int out_flag_cap, int64_t* out_len);
int su2g_prepare_input_vector(su2g_tensor ul, su2g_tensor ur, double* out, int mode, void* stream);

/* ------------------------------------------------------- measurement -- */
/* tensor_su2::take_trace (tensor_su2.cpp:720-742): the sum of the traces of
 * the blocks of equal spins of a 2-leg tensor (device data; no (2j+1)
 * weight). */
int su2g_take_trace(su2g_tensor t, double* out, void* stream);
/* tensor_su2::ss_inner_prod (tensor_su2.cpp:687-715): sum over the blocks
 * stored in a of their element overlap with b's, weighted by
 * sqrt(2j_2+1)/sqrt(2j_0+1) for 3-leg operators; a and b of one structure,
 * every block of a stored in b.  Both desc NULL (operators never built): 0. */
int su2g_ss_inner_prod(su2g_tensor a, su2g_tensor b, double* out, void* stream);
/* tensor_su2::multiply_singular_value(leg, w) (tensor_su2.cpp:359-384), in
 * place on device data: each multiplet of leg `leg` scaled by its weight,
 * w (host) laid out sector by sector in the leg's order, nw >= the leg's
 * multiplets. */
int su2g_multiply_singular_value(const int* desc, const int* flag, double* data, int leg, const double* w, int64_t nw,
                                 void* stream);
/* dmrg_su2::mea_enr (dmrg_su2_omp_mea_enr.cpp:194-242): the energy at the
 * centre bond from the environments the measurement run builds,
 *   [tr hl + tr(W hr W) + sum_k coef[k] ss_inner_prod(left[k], right[k])] / sum_i ww[i]^2,
 * hl = hh[ns/2-1], hr = hh[ns/2] (not scaled; W = the weights ww on both of
 * its legs, nww >= their multiplets; the denominator sums all nww), the pairs
 * in mea_enr's loop order (couplings with coup, plaquettes with -qdelta).
 * parts (optional, 4 doubles): tr hl, tr(W hr W), the pair sum, sum ww^2.
 * hr is left unchanged (mea_enr scales it in place). */
int su2g_mea_enr(su2g_tensor hl, su2g_tensor hr, const double* ww, int64_t nww, int npairs, const su2g_tensor* left,
                 const su2g_tensor* right, const double* coef, double* energy, double* parts, void* stream);

/* -------------------------------------------------------- checkpoints -- */
/* The engine's checkpoint files (dmrg_su2::save_mps2 / read_mps,
 * save_enr / read_enr, save_ww / read_ww; dmrg_su2_omp.cpp:864-1242), for
 * resuming a run and for serving checkpoints.  Host files, device tensors.
 * File names as the engine builds them, in the current directory:
 *   SU2G_CKPT_MPS_DAT  uu-<ns>-<dcut>-<totspin>-<ky>-<exc>-<pos>.dat
 *   SU2G_CKPT_MPS_BIN  uu-<ns>-<dcut>-<totspin>-<ky>-<exc>-<pos>.bin
 *   SU2G_CKPT_ENR      enr-<ns>-<dcut>-<totspin>-<ky>-<exc>.dat   (pos unused)
 *   SU2G_CKPT_WW       ww-<ns>-<dcut>-<totspin>-<ky>-<exc>-<pos>.bin (the engine uses pos = ns/2) */
#define SU2G_CKPT_MPS_DAT 0
#define SU2G_CKPT_MPS_BIN 1
#define SU2G_CKPT_ENR 2
#define SU2G_CKPT_WW 3
int su2g_checkpoint_name(int kind, int ns, int dcut, int totspin, int ky, int exc, int pos, char* buf, int cap);
/* One site's MPS tensor (device data) to its .dat (structure as text) and
 * .bin (block flags, reduced blocks, then the canonical CG part of each stored
 * block) files, byte for byte as save_mps2 writes them. */
int su2g_mps_save(const char* dat_path, const char* bin_path, su2g_tensor t, void* stream);
/* read_mps for one site: the structure and flags (host only), then the
 * reduced blocks into out (device, at most out_cap doubles).  Each block's CG
 * part must be proportional to the canonical one (the engine writes it
 * exactly); the block is rescaled by the ratio.  Missing or malformed files
 * give SU2G_EIO. */
int su2g_mps_load_layout(const char* dat_path, const char* bin_path, int* out_desc, int out_desc_cap, int* out_flag,
                         int out_flag_cap, int64_t* out_len);
int su2g_mps_load(const char* dat_path, const char* bin_path, double* out, int64_t out_cap, void* stream);
/* save_enr: appends one value with 16 significant digits (the engine writes
 * gs_enr, its eigenvalue with the -1000 shift where it applies); enr_read
 * returns every value of the file in order (read_enr keeps the last one and
 * adds 1000).  *count = values in the file. */
int su2g_enr_append(const char* path, double value);
int su2g_enr_read(const char* path, double* values, int cap, int* count);
/* save_ww / read_ww: raw doubles (host); *nread = doubles actually read. */
int su2g_ww_save(const char* path, const double* ww, int64_t n);
int su2g_ww_load(const char* path, double* ww, int64_t n, int64_t* nread);

/* Failure detection of the device waits, without a fault: runs the split
 * GEMM's bounded mbarrier wait on a barrier nothing arrives at, giving up
 * after `iterations` polls (> 0).  Returns SU2G_ETIMEOUT when the wait gave
 * up, as it must (the context stays usable), SU2G_OK if it completed. */
int su2g_selftest_bounded_wait(long long iterations, void* stream);

/* ------------------------------------------------------------ Lanczos -- */
/* Ground state of the plan's H_eff by the reference's Lanczos scheme
 * (lanczos_su2::lanczos1, lanczos_su2.cpp:125-195, driven as in
 * dmrg_su2::lanczos_solve_eigenvector_idmrg, dmrg_su2.cpp:527-540): at most
 * mlanc Krylov vectors, full reorthogonalisation, tridiagonal eigenproblem,
 * eigenvector check every 4 steps with early exit.  psi (device) is the start
 * vector on entry and the normalised ground state on exit; *energy receives
 * the eigenvalue (without the reference's -1000 print offset); *nmatvec, if
 * not NULL, the number of H_eff applications.  Each Lanczos step (matvec,
 * orthogonalisation, normalisation, every scalar on the device) runs as a CUDA
 * graph captured on the plan's first solve and replayed by later ones; the
 * host reads back the step's coefficients only (one copy per step). */
int su2g_lanczos(su2g_heff_plan* plan, double* psi, int mlanc, double* energy, int* nmatvec, void* stream);

/* -------------------------------------------------------------- BLAS-1 -- */
/* tensor_su2 vector algebra (tensor_su2.cpp:106-260, 324-357, 663-685) on
 * packed device vectors of n doubles.  Reductions are deterministic. */
int su2g_vec_dot(const double* x, const double* y, int64_t n, double* result, void* stream);
int su2g_vec_axpy(double alpha, const double* x, double* y, int64_t n, void* stream);
int su2g_vec_scale(double alpha, double* x, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SU2G_H */
