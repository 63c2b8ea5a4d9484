// qs_adjoint.h — observables and adjoint gradients (host entry points).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "qs_internal.h"

namespace qs {

// <a|b> into out2[0..1] (device), FP64; scratch holds up to 4096 partial pairs.
int inner_product(const void* a, int pa, const void* b, int pb, int n, cudaStream_t s, int sms, double* scratch,
                  double* out2);

int expval_pauli(const void* psi, int prec, int n, const qs_pauli_term* terms, size_t nt, cudaStream_t s, int sms,
                 double* value, std::string* msg);

int adjoint_gradient(void* state, int n, int prec, int arith, const qs_param_gate* gates, size_t m,
                     const double* params, size_t np, const qs_pauli_term* terms, size_t nt, cudaStream_t s, int sms,
                     double* energy, double* grad, size_t* err, std::string* msg);

}  // namespace qs
