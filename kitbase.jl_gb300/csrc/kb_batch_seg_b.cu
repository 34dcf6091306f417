// Instantiations of the fused FP32 batch segment kernel (kb_batch.cuh), split
// across translation units so that they compile in parallel.
#include "kb_batch.cuh"

namespace kb {

void seg_variants_b(std::vector<SegVariant>& out) {
  out.push_back({32, 128, (const void*)k_batch_seg<32, 128>, seg_smem<32, 128>, seg_smem_max<32, 128>()});
  out.push_back({32, 256, (const void*)k_batch_seg<32, 256>, seg_smem<32, 256>, seg_smem_max<32, 256>()});
}

}  // namespace kb
