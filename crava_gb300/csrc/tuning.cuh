// Tuning table lookups (see tuning.cu).
#pragma once

namespace cg {
int tune_get(int key, int n, int dflt);
}
