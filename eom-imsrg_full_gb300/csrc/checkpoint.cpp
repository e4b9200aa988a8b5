// checkpoint.cpp -- the Magnus flow with the reference's Omega checkpoints.
//
// magnus_decouple (IMSRG_MAGNUS.f90:15-128) with checkpointing on: before
// the Magnus step of every step count divisible by chk (:102-109) it writes
// Omega(s) with write_omega_checkpoint (basic_IMSRG.f90:3132-3225): the
// vectorize vector as an unformatted stream, the file named by the run prefix
// and s, and the file written 12 (eMax = 14: 4) units of s earlier removed.
// At the start it looks for a checkpoint with read_omega_checkpoint
// (:3228-3312): s from 95.5 down to above 1.0 in steps of 0.5, the first
// (largest s) file found wins.  With one, the flow restarts (:79-96):
// HS = BCH(Omega, H), the generator of HS, s = sx, steps = nint(sx/ds), and
// the first write that falls due afterwards is skipped.  The reference's
// chk rule (:56-62) and ds rule (:45-51) are imsrg_gpu_magnus_rules.
//
// The step itself is the host-driven sequence of imsrg_gpu_magnus_decouple_gen
// or one graph launch as imsrg_gpu_magnus_decouple_graph, so a restarted flow
// takes the uninterrupted one's steps.  Omega comes back from the file up to
// its diagonal rounding residue: vectorize keeps the upper triangles, and
// repackage writes a square array's diagonal as herm x the stored value
// (basic_IMSRG.f90:3906-3911), which flips the sign of the residue (about
// 1e-25) that the flow leaves on the diagonals of the anti-Hermitian Omega.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "internal.h"

namespace {

int emax_of(const imsrg_basis *b) {
  int e = 0;
  for (int a = 0; a < b->norb; a++) e = std::max(e, 2 * b->nn[a] + b->ll[a]);
  return e;
}

// write_omega_checkpoint and read_omega_checkpoint do nothing for run
// prefixes starting with 'testcase' (basic_IMSRG.f90:3144, :3241).
bool testcase(const char *prefix) { return std::strncmp(prefix, "testcase", 8) == 0; }

std::string chk_name(const char *dir, const char *prefix, double s) {
  char buf[1024];
  if (imsrg_gpu_checkpoint_name(dir, prefix, s, buf, (int)sizeof(buf)) != IMSRG_OK) return std::string();
  return std::string(buf);
}

bool file_exists(const std::string &path) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fclose(f);
  return true;
}

// write_omega_checkpoint (basic_IMSRG.f90:3132-3225) without the resubmission
// hook: Omega at s, then the checkpoint of s - 12 (eMax 14: s - 4) removed.
int write_checkpoint(const imsrg_op *G, const char *dir, const char *prefix, double s, int emax) {
  if (testcase(prefix)) return IMSRG_OK;
  const std::string path = chk_name(dir, prefix, s);
  if (path.empty()) return IMSRG_ERR_INVALID;
  IMSRG_TRY(imsrg_gpu_op_save(G, path.c_str()));
  const std::string old = chk_name(dir, prefix, emax == 14 ? s - 4.0 : s - 12.0);
  if (!old.empty() && file_exists(old)) std::remove(old.c_str());
  return IMSRG_OK;
}

// read_omega_checkpoint (basic_IMSRG.f90:3228-3312): true and sx when a file
// was found and loaded into G.
int read_checkpoint(imsrg_op *G, const char *dir, const char *prefix, bool *found, double *sx) {
  *found = false;
  if (testcase(prefix)) return IMSRG_OK;
  for (double s = 95.5; s > 1.0; s -= 0.5) {
    const std::string path = chk_name(dir, prefix, s);
    if (path.empty() || !file_exists(path)) continue;
    IMSRG_TRY(imsrg_gpu_op_load(G, path.c_str()));
    *found = true;
    *sx = s;
    return IMSRG_OK;
  }
  return IMSRG_OK;
}

int generator(imsrg_op *HS, imsrg_op *DG, int gen, int precision) {
  if (gen == IMSRG_GEN_WHITE) return imsrg_gpu_build_gs_white(HS, DG);
  if (gen == IMSRG_GEN_ATAN) return imsrg_gpu_build_gs_atan(HS, DG);
  return imsrg_gpu_build_gs_w2(HS, DG, precision);
}

void trace_row(double *trace, int k, double s, double e0, double emp2) {
  if (!trace) return;
  double *t = trace + 5 * k;
  t[0] = k;
  t[1] = s;
  t[2] = e0;
  t[3] = e0 + emp2;
  t[4] = std::fabs(emp2);
}

}  // namespace

extern "C" {

int imsrg_gpu_magnus_rules(const imsrg_basis_t *b, double lawson_beta, double *ds, int *chk) {
  if (!b) return IMSRG_ERR_INVALID;
  const int emax = emax_of(b);
  if (ds) *ds = lawson_beta < 6.0 ? 0.5 : 0.1;
  if (chk) *chk = emax == 14 ? 4 : (emax > 14 ? 1 : 24);
  return IMSRG_OK;
}

int imsrg_gpu_magnus_decouple_checkpoint(imsrg_op_t *HS, imsrg_op_t *G, int gen, double s_max, double ds,
                                         int max_steps, int precision, int use_graph, const char *dir,
                                         const char *prefix, int chk, double *trace, int *steps_out, int *ncomm,
                                         double *s_restart) {
  if (!HS || !G || !HS->b || HS->b != G->b || !HS->d || !G->d) return IMSRG_ERR_INVALID;
  if (gen != IMSRG_GEN_WHITE && gen != IMSRG_GEN_ATAN && gen != IMSRG_GEN_W2) return IMSRG_ERR_INVALID;
  if (use_graph && gen != IMSRG_GEN_WHITE) return IMSRG_ERR_INVALID;  // the step graph holds build_gs_white
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  if (ds <= 0.0 || max_steps < 0) return IMSRG_ERR_INVALID;
  const bool checkpointing = dir && prefix;
  imsrg_basis *b = HS->b;
  const int emax = emax_of(b);
  if (chk <= 0) IMSRG_TRY(imsrg_gpu_magnus_rules(b, 0.0, nullptr, &chk));
  if (s_restart) *s_restart = -1.0;
  imsrg_op *H0, *DG, *X0, *X1;
  IMSRG_TRY(imsrg::flow_tmp_ops(b, &H0, &DG, &X0, &X1));

  // magnus_decouple's set-up (IMSRG_MAGNUS.f90:31-36): DG = eta(HS), H = HS
  double s = 0.0, e0 = 0.0, emp2 = 0.0;
  if (use_graph) {
    IMSRG_TRY(imsrg::flow_graph_begin(HS, G, precision, ds, &e0, &emp2));
  } else {
    IMSRG_CUDA_TRY(cudaMemsetAsync(G->d, 0, b->nfull * sizeof(double), b->stream));
    IMSRG_CUDA_TRY(cudaMemsetAsync(DG->d, 0, b->nfull * sizeof(double), b->stream));
    G->herm = -1;
    DG->herm = -1;
    IMSRG_TRY(generator(HS, DG, gen, precision));
    IMSRG_TRY(imsrg_gpu_op_copy(HS, H0));
    IMSRG_TRY(imsrg_gpu_op_mbpt2(HS, &emp2));
    IMSRG_TRY(imsrg_gpu_op_get_e0(HS, &e0));
  }
  bool restart = false, first = false;
  double sx = 0.0;
  if (checkpointing) IMSRG_TRY(read_checkpoint(G, dir, prefix, &restart, &sx));
  int steps = 0, nct = 0;
  double crit = 10.0;
  if (!restart) {
    crit = std::fabs(emp2);
    trace_row(trace, 0, s, e0, emp2);
  } else {
    // checkpoint restart (IMSRG_MAGNUS.f90:79-96)
    G->herm = -1;
    int nb = 0;
    IMSRG_TRY(imsrg_gpu_bch_expand(HS, G, H0, precision, &nb));
    nct += nb;
    IMSRG_TRY(generator(HS, DG, gen, precision));
    s = sx;
    if (use_graph) IMSRG_TRY(imsrg::flow_graph_set_s(b, s));
    steps = (int)std::lround(sx / ds);
    first = true;
    if (s_restart) *s_restart = sx;
  }
  while (crit > 1e-6 && s < s_max - 1e-12 && steps < max_steps) {
    steps++;
    if (checkpointing && steps % chk == 0) {
      if (first) first = false;
      else IMSRG_TRY(write_checkpoint(G, dir, prefix, s, emax));
    }
    if (use_graph) {
      int nc = 0, st = IMSRG_OK;
      IMSRG_TRY(imsrg::flow_graph_launch(b));
      IMSRG_TRY(imsrg::flow_graph_finish(b, &s, &e0, &emp2, &nc, &st));
      nct += nc;
      if (st != IMSRG_OK) {
        if (steps_out) *steps_out = steps;
        if (ncomm) *ncomm = nct;
        return st;
      }
    } else {
      int nm = 0, nb = 0;
      IMSRG_TRY(imsrg_gpu_magnus_expand(DG, G, precision, &nm));
      IMSRG_TRY(imsrg_gpu_euler_step(G, DG, &s, ds));
      const int st = imsrg_gpu_bch_expand(HS, G, H0, precision, &nb);
      nct += nm + nb;
      if (st != IMSRG_OK) {
        if (steps_out) *steps_out = steps;
        if (ncomm) *ncomm = nct;
        return st;
      }
      IMSRG_TRY(generator(HS, DG, gen, precision));
      IMSRG_TRY(imsrg_gpu_op_mbpt2(HS, &emp2));
      IMSRG_TRY(imsrg_gpu_op_get_e0(HS, &e0));
    }
    if (!std::isfinite(e0) || !std::isfinite(emp2)) return IMSRG_ERR_NONFINITE;
    crit = std::fabs(emp2);
    trace_row(trace, steps, s, e0, emp2);
  }
  if (steps_out) *steps_out = steps;
  if (ncomm) *ncomm = nct;
  return IMSRG_OK;
}

}  // extern "C"
