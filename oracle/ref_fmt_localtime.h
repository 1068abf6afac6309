// Force-included into the reference build (oracle/build_ref.sh). fmt 12 removed
// fmt::localtime, which the reference CLI calls once to stamp its result file; this
// stand-in forwards to the C library so that the unmodified sources compile.
#pragma once
#ifdef __cplusplus
#include <ctime>
namespace fmt { inline namespace ref_shim { inline std::tm localtime(std::time_t t) { std::tm r{}; localtime_r(&t, &r); return r; } } }
#endif
