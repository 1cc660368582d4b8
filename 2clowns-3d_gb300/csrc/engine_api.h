// engine_api.h -- host-side entry points of the batched BiCGSTAB engine.
#pragma once

#include <cuda_runtime.h>

#include "clowns_gpu.h"

namespace clowns {

struct MemberIn;

size_t engine_workspace_bytes(int M, const int* n, int mixed);
// variant 0: PCGPME (pcgpme_para.F90); 2: PCGPME_WILL's iteration (pcgpme_2DH.f90:
// BETA = C1 / (AMU RQ), eps and iter taken as given, iter >= 1).
int engine_solve_plain(int M, const MemberIn* ins, double eps, double parm, int iter, void* work,
                       size_t work_bytes, cudaStream_t s, clowns_solve_info* info, int variant = 0);
// FP64 recursive residual r of a single-system solve left in its workspace.
double* engine_residual_ptr(void* work, int n);
int engine_solve_mixed(int M, const MemberIn* ins, double eps, double parm, double inner_tol,
                       int inner_max, int max_outer, void* work, size_t work_bytes, cudaStream_t s,
                       clowns_solve_info* info);
int engine_setup_export(const MemberIn& in, double parm, double* al_s, int* ll_s, double* d_s,
                        double* b_s, int na_out, void* work, size_t work_bytes, cudaStream_t s);
int engine_apply_pm_a(const MemberIn& in, double parm, const double* x, double* y, void* work,
                      size_t work_bytes, cudaStream_t s);
void release_all_graphs();
int engine_tuned_shape(long nv, int prec, int single, int* mode, int* block, int* grid, int* minb, int* fuse);
long engine_row_space(int M, const int* n, int mixed);
long engine_last_launches();
// Test hook: the next plain solve's cooperative loop kernel waits at most
// `limit` polls per device-wide wait and its block `absent` leaves at once.
void engine_arm_wait_fault(long limit, int absent);

}  // namespace clowns
