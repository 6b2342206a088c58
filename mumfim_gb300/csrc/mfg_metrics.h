// Structured metrics sink of the C ABI (mfg_metrics.cpp).
#ifndef MFG_METRICS_H
#define MFG_METRICS_H

#include <string>

namespace mfg {
// True when records are being written (a file is set).
bool metrics_enabled();
// Appends {"t": <unix seconds>, <fields>} as one line; `fields` is a comma
// separated list of JSON members.
void metrics_write(const std::string& fields);
double wall_seconds();
std::string json_escape(const char* s);
}  // namespace mfg

#endif
