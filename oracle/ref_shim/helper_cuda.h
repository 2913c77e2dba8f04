// Stand-in for the CUDA Samples header the reference includes
// (src/cochlea.cu:28, include/cochlea.cuh:27).  The reference's device code
// uses nothing from it; only the reference cubin build includes this file.
#pragma once
