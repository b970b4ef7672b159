// Remap table (internal): the rows (iD, jD, iS, jS, w) of a mapping-table
// file in host memory, 1-based grid indices, in file order.  Filled by the
// Jones-99 (remap.cu) and bilinear (bilin.cu) generators and by the reader.
#pragma once
#include <stdint.h>

#include <vector>

struct dccm_remap_table {
  std::vector<int32_t> iD, jD, iS, jS;
  std::vector<double> w;
};
