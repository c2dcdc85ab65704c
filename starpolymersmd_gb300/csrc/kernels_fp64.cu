// FP64 reference-parity instantiation. Built with -fmad=false so every
// multiply and add rounds separately, in the reference's order.
#define SMPC_REAL double
#define SMPC_FAST_F32 0
#define SMPC_COLLIDE_NT 128
#define SMPC_COLLIDE_CT 64
#define SMPC_COLLIDE_CAP 768
#define SMPC_BIN_NT 256
#define SMPC_MD_NT 256
#define SMPC_MD_MPT 4
#include "kernels_impl.cuh"

namespace smpc {
// solvent slots per binning block: FP64 blocks hold two records per thread
// in flight (k_fluid_bin), FP32 blocks four
int fluid_slots_per_tile(bool fp64) { return fp64 ? 2048 : 4096; }
int temperature_cells_per_tile() { return 512; }
int md_max_monomers() { return SMPC_MD_NT * SMPC_MD_MPT; }
int pmd_block_count(int n_beads) { return (n_beads + PMD_NT - 1) / PMD_NT; }
}  // namespace smpc
