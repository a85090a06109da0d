// Opt-in per-kernel-class event timing (see prof.cu).
#pragma once
#include "common.cuh"

namespace qr {
enum ProfKind { PK_ZGEMM = 0, PK_JACOBI64 = 1, PK_JACOBI32 = 2, PK_QR = 3, PK_ENV = 4, PK_ZGEMM_SPLIT = 5, PK_JACOBI_DF = 6, PK_ZGEMM_DF = 7, PK_COUNT = 8 };
bool prof_on();
// returns a record index (or -1 when profiling is off); pair with prof_end on the same stream
int prof_begin(cudaStream_t s, int kind, double flops, double bytes);
void prof_end(cudaStream_t s, int idx);
// set the work of a record after the fact (flops/bytes known only once the launches ran); units
// >= 0 replaces the record's unit count (1 by default: one launch; the Jacobi stages count the
// sweeps that ran)
void prof_account(int idx, double flops, double bytes, long units = -1);
}  // namespace qr
