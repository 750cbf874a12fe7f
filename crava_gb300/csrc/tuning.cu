// Tuning table: launch variants chosen per transform length or stack count.
// Defaults are built in (measured on GB300); cg_tune_set overrides them, and
// the environment variables CRAVA_COLS_MINB, CRAVA_COLS_PIPE, CRAVA_BIN_MINB,
// CRAVA_ROWS_KERNEL, CRAVA_FUSED_Y, CRAVA_BIN_FORM, CRAVA_XY_PLANE, CRAVA_COLS_SHAPE and CRAVA_BIN_RUNS override both (used by
// ad-hoc sweeps).
#include <cstdlib>
#include <map>
#include <mutex>

#include "common.cuh"
#include "tuning.cuh"

namespace cg {

namespace {
std::mutex g_mu;
std::map<long, int> g_table;  // (key << 32) | n  ->  value, n = 0 for "every n"
const char *env_name(int key)
{
  switch (key) {
    case CG_TUNE_COLS_MINB: return "CRAVA_COLS_MINB";
    case CG_TUNE_COLS_PIPE: return "CRAVA_COLS_PIPE";
    case CG_TUNE_BIN_MINB: return "CRAVA_BIN_MINB";
    case CG_TUNE_ROWS_KERNEL: return "CRAVA_ROWS_KERNEL";
    case CG_TUNE_FUSED_Y: return "CRAVA_FUSED_Y";
    case CG_TUNE_BIN_FORM: return "CRAVA_BIN_FORM";
    case CG_TUNE_XY_PLANE: return "CRAVA_XY_PLANE";
    case CG_TUNE_COLS_SHAPE: return "CRAVA_COLS_SHAPE";
    case CG_TUNE_BIN_RUNS: return "CRAVA_BIN_RUNS";
    default: return nullptr;
  }
}
bool valid_value(int key, int value)
{
  return (key == CG_TUNE_COLS_MINB && (value >= 2 && value <= 4)) ||
         (key == CG_TUNE_COLS_PIPE && (value >= 0 && value <= 5)) ||
         (key == CG_TUNE_BIN_MINB && (value == 1 || (value >= 4 && value <= 6))) ||
         (key == CG_TUNE_ROWS_KERNEL && (value == 0 || value == 1)) ||
         (key == CG_TUNE_FUSED_Y && (value >= 0 && value <= 2 || (value >= 4 && value <= 4096 && value % 2 == 0))) ||
         (key == CG_TUNE_BIN_FORM && (value == 0 || value == 1)) ||
         (key == CG_TUNE_XY_PLANE && (value == 0 || value == 1)) ||
         (key == CG_TUNE_COLS_SHAPE && (value >= 0 && value <= 3)) ||
         (key == CG_TUNE_BIN_RUNS && (value >= 0 && value <= 8));
}
}  // namespace

int tune_get(int key, int n, int dflt)
{
  const char *en = env_name(key);
  if (en) {
    const char *e = getenv(en);
    if (e && *e && valid_value(key, atoi(e))) return atoi(e);  // an invalid value is ignored
  }
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(((long)key << 32) | (unsigned)n);
  if (it != g_table.end()) return it->second;
  it = g_table.find((long)key << 32);
  if (it != g_table.end()) return it->second;
  return dflt;
}

}  // namespace cg

using namespace cg;

extern "C" int cg_tune_set(int key, int n, int value)
{
  if (key < CG_TUNE_COLS_MINB || key > CG_TUNE_BIN_RUNS || n < 0) { set_error("cg_tune_set: bad key or n"); return CG_ERR_ARG; }
  if (!valid_value(key, value)) { set_error("cg_tune_set: value %d not valid for key %d", value, key); return CG_ERR_ARG; }
  std::lock_guard<std::mutex> lk(g_mu);
  g_table[((long)key << 32) | (unsigned)n] = value;
  return CG_OK;
}

extern "C" int cg_tune_clear(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  g_table.clear();
  return CG_OK;
}

extern "C" int cg_tune_get(int key, int n)
{
  switch (key) {
    case CG_TUNE_COLS_MINB: return tune_get(key, n, n <= 256 ? 3 : 2);
    case CG_TUNE_COLS_PIPE: return tune_get(key, n, n == 256 ? 2 : 3);  // register-direct at 256, four-step elsewhere
    case CG_TUNE_BIN_MINB: return tune_get(key, n, n <= 5 ? 6 : 1);
    case CG_TUNE_ROWS_KERNEL: return tune_get(key, n, 1);  // four-step
    case CG_TUNE_FUSED_Y: return tune_get(key, n, 0);
    case CG_TUNE_BIN_FORM: return tune_get(key, n, 1);  // information form
    case CG_TUNE_XY_PLANE: return tune_get(key, n, 0);
    case CG_TUNE_COLS_SHAPE: return tune_get(key, n, 0);
    case CG_TUNE_BIN_RUNS: return tune_get(key, n, 0);
    default: set_error("cg_tune_get: bad key"); return CG_ERR_ARG;
  }
}
