// Mypool.h (stand-in) — TEST INFRASTRUCTURE ONLY: the TBB memory pool is not
// used by the kernel functions of particle.cpp.
#pragma once
