// FP32 fast-path instantiation: float4 state, int64 fixed-point cell sums.
#define SMPC_REAL float
#define SMPC_FAST_F32 1
#define SMPC_COLLIDE_NT 256
#define SMPC_COLLIDE_CT 128
#define SMPC_COLLIDE_CAP 1408
#define SMPC_BIN_NT 256
#define SMPC_MD_NT 1024
#define SMPC_MD_MPT 1
#include "kernels_impl.cuh"

namespace smpc {
// Variant tables (index 0 is the default shape). The names read
// threads x cells-per-tile / staging capacity / gathers in flight.
int bin_variant_count() { return 4; }
int collide_variant_count() { return 12; }
int md_variant_count() { return 5; }
int collide_variant_cells(int v) {
  switch (v) {
    case 2: case 3: case 5: case 7: case 8: case 9: case 10: case 11: return 64;
    case 4: return 256;
    default: return 128;
  }
}
const char* bin_variant_name(int v) {
  static const char* n[] = {"256t x4", "256t x2", "256t x8", "128t x8"};
  return v >= 0 && v < 4 ? n[v] : "?";
}
const char* collide_variant_name(int v) {
  static const char* n[] = {"256t 128c cap1408 g4", "256t 128c cap1408 g8", "128t 64c cap704 g4",
                            "128t 64c cap704 g8", "512t 256c cap2816 g4",
                            "128t 64c cap704 cp.async", "256t 128c cap1408 cp.async",
                            "128t 64c cap736 cp.async", "128t 64c cap768 cp.async",
                            "160t 64c cap704 cp.async", "192t 64c cap704 cp.async",
                            "256t 64c cap704 cp.async"};
  return v >= 0 && v < 12 ? n[v] : "?";
}
int pmd_variant_count() { return 4; }
int pmd_variant_lanes(int v) {
  static const int lanes[] = {8, 4, 16, 8};
  return v >= 0 && v < 4 ? lanes[v] : 8;
}
int pmd_variant_list_blocks_per_sm(int v) { return v == 3 ? 8 : 4; }
const char* pmd_variant_name(int v) {
  static const char* n[] = {"8 lanes/bead, lists 4 blocks/SM", "4 lanes/bead, lists 4 blocks/SM",
                            "16 lanes/bead, lists 4 blocks/SM", "8 lanes/bead, lists 8 blocks/SM"};
  return v >= 0 && v < 4 ? n[v] : "?";
}
const char* md_variant_name(int v) {
  static const char* n[] = {"1024t 1/thread", "512t 2/thread", "1024t lanes/bead, largest first",
                            "1024t big + 512t small side by side, lanes/bead",
                            "cluster of SMs per replica (few replicas; else 1024t 1/thread)"};
  return v >= 0 && v < 5 ? n[v] : "?";
}
}  // namespace smpc
