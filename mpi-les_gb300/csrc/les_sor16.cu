// les_sor16.cu -- the fused SOR sweep (les_sor.cu) on 16-column tiles: 56 interior i
// cells per CTA, two CTAs per SM, for narrow domains (batch members, and small domains
// alone when the tuner finds them faster), whole march or k chunks, with a uniform cn1
// (the only form the register kernel is instantiated for here).
#include "les_sor_kern.cuh"

namespace {

template <int NY, int D, bool KC>
void launch16_kc(const LesDom &d, const SorArgs &a, const CUtensorMap *tp, const CUtensorMap *tr, cudaStream_t s) {
  if (tp && tr) launch_tma_kc<16, NY, D, KC>(d, a, *tp, *tr, s);
  else launch_reg_kc<16, NY, KC>(d, a, 0, s);
}
template <int NY, int D>
void launch16(const LesDom &d, const SorArgs &a, const CUtensorMap *tp, const CUtensorMap *tr, cudaStream_t s) {
  if (a.nchunk > 1) launch16_kc<NY, D, true>(d, a, tp, tr, s);
  else launch16_kc<NY, D, false>(d, a, tp, tr, s);
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
