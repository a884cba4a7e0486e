// env.cpp - environment knobs with the reference's parsing rules
// (IPT_C_GPU/src/ipt_cuda.cu:18-73): unset/empty => default; numbers that do
// not parse, are negative or non-finite => default; flags are false only for
// "0", "false", "FALSE", "no", "NO".
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace iptgb {

double env_double(const char *name, double default_value)
{
    const char *raw = getenv(name);
    if (raw == nullptr || raw[0] == '\0') {
        return default_value;
    }
    char *end = nullptr;
    const double v = strtod(raw, &end);
    if (end == raw || v < 0.0 || !std::isfinite(v)) {
        return default_value;
    }
    return v;
}

int env_int(const char *name, int default_value)
{
    const char *raw = getenv(name);
    if (raw == nullptr || raw[0] == '\0') {
        return default_value;
    }
    char *end = nullptr;
    const long v = strtol(raw, &end, 10);
    if (end == raw || v < 0 || v > INT_MAX) {
        return default_value;
    }
    return (int)v;
}

int env_flag(const char *name, int default_value)
{
    const char *raw = getenv(name);
    if (raw == nullptr || raw[0] == '\0') {
        return default_value;
    }
    if (strcmp(raw, "0") == 0 || strcmp(raw, "false") == 0 || strcmp(raw, "FALSE") == 0 ||
        strcmp(raw, "no") == 0 || strcmp(raw, "NO") == 0) {
        return 0;
    }
    return 1;
}

}  // namespace iptgb
