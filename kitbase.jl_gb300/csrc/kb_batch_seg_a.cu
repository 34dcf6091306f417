// Instantiations of the fused FP32 batch segment kernel (kb_batch.cuh), split
// across translation units so that they compile in parallel.
#include "kb_batch.cuh"

namespace kb {

void seg_variants_a(std::vector<SegVariant>& out) {
  out.push_back({8, 64, (const void*)k_batch_seg<8, 64>, seg_smem<8, 64>, seg_smem_max<8, 64>()});
  out.push_back({16, 64, (const void*)k_batch_seg<16, 64>, seg_smem<16, 64>, seg_smem_max<16, 64>()});
  out.push_back({16, 128, (const void*)k_batch_seg<16, 128>, seg_smem<16, 128>, seg_smem_max<16, 128>()});
  out.push_back({16, 256, (const void*)k_batch_seg<16, 256>, seg_smem<16, 256>, seg_smem_max<16, 256>()});
}

}  // namespace kb
