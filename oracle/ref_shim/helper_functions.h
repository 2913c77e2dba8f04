// Stand-in for the CUDA Samples header the reference includes
// (src/cochlea.cu:26, include/cochlea.cuh:26).  The reference's device code
// uses nothing from it; only the reference cubin build includes this file.
#pragma once
