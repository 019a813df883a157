// Host build of the cull's work-item layout (pipeline_gb300/csrc/dpcull_internal.h:
// lay_out_items, tile_groups_of) for tests/test_item_layout.py.
#include <cstdint>
#include <vector>

#include <vector_types.h>  // uint2 and friends, as the CUDA sources see them

#include "dpcull_internal.h"

// scenes i = 0..n-1 with n_tiles[i] tiles and n_vgroups[i] view groups: fills n_big[i] and
// item_begin[i]; returns the launch's item count.
extern "C" uint32_t layout_items(size_t n, const uint32_t* n_tiles, const uint32_t* n_vgroups,
                                 uint32_t item_tiles, uint64_t tail, uint32_t* n_big, uint32_t* item_begin)
{
  std::vector<dpcull::CullScene> sc(n);
  for (size_t i = 0; i < n; ++i) {
    sc[i] = dpcull::CullScene{};
    sc[i].n_tiles = n_tiles[i];
    sc[i].n_vgroups = n_vgroups[i];
  }
  const uint32_t items = dpcull::lay_out_items(sc.data(), n, item_tiles, tail);
  for (size_t i = 0; i < n; ++i) {
    n_big[i] = sc[i].n_big;
    item_begin[i] = sc[i].item_begin;
  }
  return items;
}

extern "C" uint32_t groups_of(uint32_t n_tiles, uint32_t n_big, uint32_t item_tiles)
{
  return dpcull::tile_groups_of(n_tiles, n_big, item_tiles);
}

extern "C" uint32_t tiles_for(uint64_t tile_groups, int sm_count) { return dpcull::item_tiles_for(tile_groups, sm_count); }
extern "C" uint64_t tail_for(int sm_count) { return dpcull::tail_units(sm_count); }
