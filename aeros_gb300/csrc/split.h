// split.h -- split-precision (Ozaki) Legendre contraction on the tensor cores.
#pragma once
#include "aeros_internal.h"

namespace aeros {

struct SplitCtx;

// Build the sliced Legendre tables for geometry g; `max_rows` bounds the
// Fourier rows per call.
int split_create(const Geometry &g, const DevTables &t, int max_rows, SplitCtx **out);
void split_destroy(SplitCtx *s);
// Same contract as launch_leg_synth_fp64 / launch_leg_anal_fp64.
int split_leg_synth(SplitCtx *s, const Ctx &c, const SynPlan &p, double2 *F, int nrow);
// The analysis runs on column groups of AnaCols (split_anal_groups: group g
// is [start[g], start[g + 1]), packed by used slots); gstart_d holds the
// ngrp + 1 starts on the device.
int split_leg_anal(SplitCtx *s, const Ctx &c, const AnaCol *cols_d, const int *gstart_d, int ngrp, const double2 *F,
                   int nrow);
std::vector<int> split_anal_groups(const std::vector<AnaCol> &cols);
// Sticky device error flag of the split kernels (1: an mbarrier wait gave up,
// 2: misaligned shared memory); read after the stream has synchronised.
int split_error(SplitCtx *s, int *flag);
// AEROS_OK, or AEROS_ERR_CUDA with the last-error text set when the flag is up.
int split_check(SplitCtx *s);
// The same check split in two, for a caller that reads several flags with one
// synchronisation: the device word (nullptr for a null context), then its status.
const int *split_err_word(const SplitCtx *s);
int split_flag_status(int flag);

// Longitude transforms of the split form as exact-digit DFT products on the
// tensor cores (split_dft.cu).  Same contracts as launch_fourier_synth /
// launch_fourier_anal; a direction whose contraction exceeds 441 is not built
// (has_* false) and keeps the FFT.  Creation returns a null context unless the
// environment sets AEROS_SPLIT_DFT=1: by default the split form's longitude
// transforms are the double-float FFTs (launch_fourier_*_df).
struct SplitDft;
int split_dft_create(const Geometry &g, SplitDft **out);
void split_dft_destroy(SplitDft *s);
bool split_dft_has_synth(const SplitDft *s);
bool split_dft_has_anal(const SplitDft *s);
int split_fourier_synth(SplitDft *s, const Ctx &c, const FsynField *fields_d, int nf, const double2 *F, int nrow);
int split_fourier_anal(SplitDft *s, const Ctx &c, const FanaField *fields_d, int nf, double2 *F, int nrow);
int split_dft_check(SplitDft *s);
const int *split_dft_err_word(const SplitDft *s);
int split_dft_flag_status(int flag);

}  // namespace aeros
