// les_sor16.cu -- the fused SOR sweep (les_sor.cu) on 16-column tiles: 56 interior i
// cells per CTA, two CTAs per SM.  Used for domains that share the GPU, whose SOR
// march is never split in k, with a uniform cn1 (the only form the register kernel is
// instantiated for here).
#include "les_sor_kern.cuh"

namespace {

template <int NY, int D>
void launch16(const LesDom &d, const SorArgs &a, const CUtensorMap *tp, const CUtensorMap *tr, cudaStream_t s) {
  if (tp && tr) launch_tma_kc<16, NY, D, false>(d, a, *tp, *tr, s);
  else launch_reg_kc<16, NY, false>(d, a, 0, s);
}

}  // namespace

void les_launch_sor_iter_nx16(const LesDom &d, const SorArgs &a, int ny, const CUtensorMap *tp,
                              const CUtensorMap *tr, cudaStream_t s) {
  // shared memory per CTA stays below half an SM's: (2 D + 2) * NY * 256 B + 6 KB
  switch (ny) {
    case 16: launch16<16, 6>(d, a, tp, tr, s); break;
    case 20: launch16<20, 6>(d, a, tp, tr, s); break;
    case 28: launch16<28, 4>(d, a, tp, tr, s); break;
    default: launch16<24, 6>(d, a, tp, tr, s); break;
  }
}
