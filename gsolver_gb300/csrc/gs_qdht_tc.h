// gs_qdht_tc.h -- mixed-precision QDHT on the tcgen05 tensor cores (split FP16 or TF32 operands,
// FP32 accumulate).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "gs_kernels.h"

namespace gs {

struct QdhtTc;

// Plan for an n_r x n_r real matrix applied to [n_r][n_t] complex float rows.
// Returns nullptr (and a message) when the grid is not supported.
QdhtTc* qdht_tc_create(int nr, int nt, cudaStream_t st, std::string* msg);
// Upload C (element (i,j) at C[i + nr*j]) and m1; builds the split hi/lo operands.
int qdht_tc_set_matrix(QdhtTc* q, const double* C, const double* m1, std::string* msg);
// Linear-step tables (position order, FP64): k(omega), HO dispersion, kt^2 and the window.
int qdht_tc_set_lstep(QdhtTc* q, const double* omega, const double* wavenum, const double* ho, const double* kt2,
                      double omega_min, double omega_max, std::string* msg);
// Nonzero (with a message) if a kernel recorded an expired wait since the last check.
int qdht_tc_check(QdhtTc* q, std::string* msg);
// Self-test of the bounded waits: a kernel waits limit_s on an mbarrier nothing arrives at,
// records the expiry as the GEMM's waits do and returns (synchronises the plan's stream).
cudaError_t qdht_tc_wait_probe(QdhtTc* q, double limit_s, long long* nlaunch);
// Y = QDHT(X) with the given mode (QDHT_PLAIN / QDHT_LSTEP / QDHT_MASKED).  Flags:
//   QTC_X_COMPACT  linear step: X's spectral-window columns are already in the compact array
//                  of qdht_tc_compact_x (X itself is not read);
//   QTC_S_COMPACT  BIGBUFFER2's window columns live in the plan's compact copy: the linear
//                  step updates it (Y is not touched) and the masked inverse reads it (X is
//                  not read); see qdht_tc_spec_copy.
//   QTC_Y_LAZY     masked inverse: leave the result in the compact array of qdht_tc_compact_y
//                  (Y is not written; qdht_tc_expand writes it when it is wanted).
enum { QTC_X_COMPACT = 1, QTC_S_COMPACT = 2, QTC_Y_LAZY = 4 };
cudaError_t qdht_tc_run(QdhtTc* q, int mode, const float* X, float* Y, const LstepArgs& L, long long* nlaunch,
                        std::string* msg, int flags = 0);
// The plan keeps compact copies of the window's columns (wide-tile plans with linear-step tables).
bool qdht_tc_has_compact(const QdhtTc* q);
// Copy BIGBUFFER2 S's window columns into the compact copy (to_compact != 0; its low parts
// zero) or back into S (the high parts).  The compact copy is a double-float pair (high, low):
// the linear step updates it with ~48 significant bits.
cudaError_t qdht_tc_spec_copy(QdhtTc* q, float* S, int to_compact, long long* nlaunch);
// The compact copy from / into an FP64 [n_r][n_t] complex array X (device or pinned host
// memory) whose column perm[p] holds position p (perm null: position order): take != 0 splits
// X's window pairs into high and low parts; take == 0 adds the low parts into X, which must
// already hold the high parts there.
cudaError_t qdht_tc_spec_ff(QdhtTc* q, double* X, const int* perm, int take, long long* nlaunch);
// The same from / into device arrays in position order: S (high parts) and lo (low parts), both
// [n_r][2 n_t] floats; take != 0 sets the compact copy from them, take == 0 writes lo over the
// whole array (the compact low parts at the window's pairs, zeros elsewhere).
cudaError_t qdht_tc_spec_dev(QdhtTc* q, float* S, float* lo, int take, long long* nlaunch);
// BIGBUFFER2's compact double-float copy itself: high and low parts, each [n_r][nc] floats
// (null when the plan keeps none)
void qdht_tc_spec_pairs(QdhtTc* q, float** sc, float** sl, int* nc);
// The compact [n_r][nc] input array of the linear-step transform and its position map (cinv[p]:
// the column of position p's (re, im) pair, or -1 outside the spectral window); null when the
// plan has no window columns (set_lstep not called, or a width outside the wide-tile path).
float* qdht_tc_compact_x(QdhtTc* q, const int** cinv, int* nc);
// The masked inverse's compact [n_r][nc] result array (same columns and position map as
// qdht_tc_compact_x; cmap[c]: the real column of compact column c, -1 in the padding), and
// its expansion into Y (zeros outside the spectral window).
const float* qdht_tc_compact_y(QdhtTc* q, int* nc, const int** cmap = nullptr);
cudaError_t qdht_tc_expand(QdhtTc* q, float* Y, long long* nlaunch, const int* run = nullptr);
// Adjoint of the QDHT_LSTEP epilogue's linear step, elementwise over [n_r][n_t]: fb = cotangent
// of FIELD (k,omega), sb of BIGBUFFER2 (in: after the step, out: before), b1b out: of
// BIGBUFFER1 (k,omega).  When the plan forms the forward's factors in double-float
// (qdht_tc_lstep_adj_ff) and sbl is given, the adjoint does the same and sb + sbl is
// BIGBUFFER2's cotangent as double-float pairs (sbl: their low parts, zero to start);
// otherwise FP32 with the epilogue's FP32 tables.
cudaError_t qdht_tc_lstep_adj(QdhtTc* q, const float* fb, float* sb, float* sbl, float* b1b, double dz,
                              long long* nlaunch);
bool qdht_tc_lstep_adj_ff(const QdhtTc* q);
void qdht_tc_destroy(QdhtTc* q);

}  // namespace gs
