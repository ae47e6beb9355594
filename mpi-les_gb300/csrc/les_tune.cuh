// les_tune.cuh -- measured tile shapes of the fused SOR sweep per size class (les_tune.cu).
#pragma once
#include <string>

#include "les_common.cuh"
#include "les_sor.cuh"

// Time the candidate shapes for domain d (alone on the GPU, or as one of many domains
// sharing it) on scratch copies of its SOR buffers, store the fastest in the class
// table and return it.  0 on success, 1 if the domain has no fused sweep to tune, < 0
// on a CUDA failure.  mem_budget bounds the scratch memory of the shared timing.
int les_tune_sor(const LesDom &d, bool shared, size_t mem_budget, SorShape *best, double *best_sec,
                 std::string *report);
// The class table: lookup returns false when the class was never tuned; storing a
// shape with nx == 0 erases the entry.
bool les_tune_lookup(int im, int jm, int km, int shared, int sms, SorShape *out);
void les_tune_store(int im, int jm, int km, int shared, int sms, SorShape sh);
