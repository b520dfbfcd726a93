// The source-group propagation kernels of geodesic.cu built with out-of-line hash-table probes: one copy of each
// probe instead of one per call site, a smaller kernel with fewer instruction-cache misses.  Where sources are small
// (tens of windows each, every phase of the kernel hot at once) this build is faster; where they are large the
// inlined probes win.  The autotuner picks per system (GeoLaunch::hashOutline); results are the same.
#define CSSG_GEO_OUTLINE 1
#include "geodesic.cu"
