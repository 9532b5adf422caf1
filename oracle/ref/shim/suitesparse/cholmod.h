/* Build shim: opaque stand-ins for the SuiteSparse types named by the xerus
 * reference headers. The dense code path used as an oracle never reaches them. */
#pragma once
#include <cstddef>
struct cholmod_common { int unused; };
struct cholmod_sparse { int unused; };
