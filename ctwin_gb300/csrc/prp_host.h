// Host helpers shared by the PRP engine, the pools and the server.
#pragma once
#include <cstddef>
#include <cstdint>

namespace ctw {

// Record an error message for ctw_last_error() and return `code`.
int fail(int code, const char *fmt, ...);

// Canonical digits (base b, 0 <= d < b) of the value of the signed digits x
// modulo N = b^D - b^{D/2} + 1, as the reference's transform::getInt.
int canonical(const int32_t *x, uint32_t b, size_t D, uint32_t *out);

// The same modulo N- = b^Dn - b^{Dn/2} - 1 (x holds Dn digits).
int canonical_minus(const int32_t *x, uint32_t b, size_t Dn, uint32_t *out);

// PRP flag (value == 1), zero flag and RES64 of canonical digits.
void res64_of(const uint32_t *c, uint32_t b, size_t D, bool &prp, bool &zero, uint64_t &r64);

}  // namespace ctw
