#pragma once
#include "stub_prelude.h"
