/* LolaCUDA kernels instantiated for LOLA_STORE_TEX32 (one translation unit per
 * storage layout so the library's kernels compile in parallel). */
#include "bp_staged.cuh"
#include "bp_batch.cuh"

LOLA_INSTANTIATE_STORAGE(LOLA_STORE_TEX32, TEX32)
