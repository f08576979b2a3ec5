// level_infor.h (stand-in) — TEST INFRASTRUCTURE ONLY: nothing of it is used by
// the kernel functions of particle.cpp.
#pragma once
