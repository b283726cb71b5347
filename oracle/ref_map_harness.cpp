/*
 * ref_map_harness.cpp -- C entry point into the reference's own genetic map
 * (geneticMap.hpp / geneticMap.cpp, compiled unmodified from the reference
 * tree by oracle/Makefile).  TEST INFRASTRUCTURE ONLY: the resulting
 * oracle/_ref/libglp_ref_map.so pins glphase_gb300/io.py's GeneticMap; it
 * never runs on the product path.
 *
 *   glpr_genetic_distances -> GeneticMap::GeneticMap (geneticMap.cpp:4-44)
 *                             on an uncompressed map file, then
 *                             GeneticLocation (46-70) and GeneticDistance
 *                             (72-79) at the given positions.
 */
#include <cstdint>
#include <stdexcept>
#include <string>

#include "geneticMap.hpp"

extern "C" {

// loc[m] = GeneticLocation(pos[m]) (cM); dist[m] = GeneticDistance(pos[m-1],
// pos[m]) (Morgans), dist[0] = 0.  Returns 0, or -1 when the reference
// throws (unreadable or malformed map, a position off the map, positions
// out of order).
int glpr_genetic_distances(const char *path, const uint32_t *pos, uint32_t n, double *loc,
                           double *dist) {
  try {
    std::string name(path);
    GeneticMap gm(name);
    for (uint32_t m = 0; m < n; ++m) {
      loc[m] = gm.GeneticLocation(pos[m]);
      dist[m] = m ? gm.GeneticDistance(pos[m - 1], pos[m]) : 0.0;
    }
  } catch (const std::exception &) {
    return -1;
  }
  return 0;
}

}  // extern "C"
