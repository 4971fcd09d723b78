// Prints the host-side sizing facts the CPU tests check: ring buffer counts per penalty set,
// arena layouts for three and five components, and the C ABI's wfg_config_t layout.
#include <cstddef>
#include <cstdio>

#include "wfa_gpu.h"
#include "wfg_internal.h"

int main() {
  using namespace wfg;
  printf("ring_buffers_4_6_2\t%d\n", wfg_ring_buffers(4, 6, 2));
  printf("ring_buffers_1_2_1\t%d\n", wfg_ring_buffers(1, 2, 1));
  printf("ring_buffers_linear_4_2\t%d\n", wfg_ring_buffers(4, 2, 0));
  printf("ring_buffers_2p_4_6_2_24_1\t%d\n", wfg_ring_buffers_2p(4, 6, 2, 24, 1));
  printf("ring_buffers_2p_4_6_2_24_2\t%d\n", wfg_ring_buffers_2p(4, 6, 2, 24, 2));
  printf("ring_buffers_2p_4_12_4_24_4\t%d\n", wfg_ring_buffers_2p(4, 12, 4, 24, 4));
  const ArenaLayout a3 = wfg_arena_layout(5, 4096, 528, 65536, 2002, 2002, 64);
  const ArenaLayout a5 = wfg_arena_layout(5, 4096, 528, 65536, 2002, 2002, 64, 5);
  printf("arena3_ring\t%lld\n", (long long)a3.ring_bytes);
  printf("arena5_ring\t%lld\n", (long long)a5.ring_bytes);
  printf("arena3_ldesc\t%lld\n", (long long)a3.ldesc_bytes);
  printf("arena5_ldesc\t%lld\n", (long long)a5.ldesc_bytes);
  printf("arena3_rdesc2\t%lld\n", (long long)a3.rdesc2_bytes);
  printf("arena5_rdesc2\t%lld\n", (long long)a5.rdesc2_bytes);
  printf("arena3_total\t%lld\n", (long long)a3.total);
  printf("arena5_total\t%lld\n", (long long)a5.total);
  printf("arena5_end\t%lld\n", (long long)(a5.rdesc2_off + a5.rdesc2_bytes));
  printf("sizeof_wfg_config_t\t%zu\n", sizeof(wfg_config_t));
  printf("offsetof_metric\t%zu\n", offsetof(wfg_config_t, metric));
  printf("offsetof_gap_opening2\t%zu\n", offsetof(wfg_config_t, gap_opening2));
  printf("offsetof_gap_extension2\t%zu\n", offsetof(wfg_config_t, gap_extension2));
  printf("max_scope\t%d\t%d\n", WFG_MAX_SCOPE, WFG_MAX_SCOPE_2P);
  return 0;
}
