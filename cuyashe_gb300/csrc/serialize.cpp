// serialize.cpp -- on-disk / wire format for keys and ciphertexts (host only).
//
// The reference keeps keys and ciphertexts as NTL objects in process memory and
// has no serialised form. Here a blob is a fixed header, the polynomials as
// little-endian 64-bit limbs and a checksum, so that a serving process can save
// its keys and resume with them, and ciphertexts can travel between processes:
//
//   offset  size       field
//   0       4          magic "CYSH"
//   4       4          u32 version (1)
//   8       4          u32 kind (CY_BLOB_*)
//   12      4          u32 n
//   16      4          u32 q_limbs (L)
//   20      4          u32 count (polynomials)
//   24      8          u64 t (0 when not a YASHE object)
//   32      4          u32 w_bits (0 when not a YASHE object)
//   36      4          u32 reserved (0)
//   40      8 L        q, L limbs
//   40+8L   8 count n L  polynomials [count][n][L], coefficients in [0, q)
//   end     8          u64 FNV-1a of every byte before it
//
// All integers little endian, independent of the host's byte order.
#include <cstring>
#include <vector>

#include "host.h"

namespace cy {

static const unsigned char kMagic[4] = {'C', 'Y', 'S', 'H'};
constexpr uint32_t kVersion = 1;
constexpr size_t kHeader = 40;

static void put32(unsigned char* p, uint32_t v) {
    for (int i = 0; i < 4; i++) p[i] = (unsigned char)(v >> (8 * i));
}
static void put64(unsigned char* p, uint64_t v) {
    for (int i = 0; i < 8; i++) p[i] = (unsigned char)(v >> (8 * i));
}
static uint32_t get32(const unsigned char* p) {
    uint32_t v = 0;
    for (int i = 0; i < 4; i++) v |= (uint32_t)p[i] << (8 * i);
    return v;
}
static uint64_t get64(const unsigned char* p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v |= (uint64_t)p[i] << (8 * i);
    return v;
}
static uint64_t fnv1a(const unsigned char* p, size_t n) {
    uint64_t h = 0xCBF29CE484222325ULL;
    for (size_t i = 0; i < n; i++) {
        h ^= p[i];
        h *= 0x100000001B3ULL;
    }
    return h;
}

static size_t blob_bytes(int n, int q_limbs, int count) {
    return kHeader + 8 * (size_t)q_limbs + 8 * (size_t)count * n * q_limbs + 8;
}

// Polynomial coefficients must be below q.
static bool coeffs_below_q(const uint64_t* polys, size_t coeffs, const uint64_t* q, int L) {
    for (size_t c = 0; c < coeffs; c++) {
        const uint64_t* x = polys + c * L;
        int w = L - 1;
        while (w >= 0 && x[w] == q[w]) w--;
        if (w < 0 || x[w] > q[w]) return false;
    }
    return true;
}

}  // namespace cy

using namespace cy;

extern "C" {

cy_status cy_serialize(uint32_t kind, int n, const uint64_t* q, int q_limbs, uint64_t t, int w_bits,
                       const uint64_t* polys, int count, void* buf, size_t len, size_t* needed) {
    if (n < 1 || q_limbs < 1 || q_limbs > CY_BLOB_MAX_LIMBS || count < 0 || !q || (count > 0 && !polys) || w_bits < 0 ||
        kind < CY_BLOB_CIPHERTEXTS || kind > CY_BLOB_KEYS)
        return set_error(CY_ERR_INVALID_ARGUMENT, "bad argument");
    const size_t bytes = blob_bytes(n, q_limbs, count);
    if (needed) *needed = bytes;
    if (!buf) return CY_OK;  // size query
    if (len < bytes) return set_error(CY_ERR_INVALID_ARGUMENT, "buffer too small");
    if (!coeffs_below_q(polys, (size_t)count * n, q, q_limbs))
        return set_error(CY_ERR_INVALID_ARGUMENT, "coefficient not in [0, q)");
    unsigned char* p = static_cast<unsigned char*>(buf);
    std::memcpy(p, kMagic, 4);
    put32(p + 4, kVersion);
    put32(p + 8, kind);
    put32(p + 12, (uint32_t)n);
    put32(p + 16, (uint32_t)q_limbs);
    put32(p + 20, (uint32_t)count);
    put64(p + 24, t);
    put32(p + 32, (uint32_t)w_bits);
    put32(p + 36, 0);
    unsigned char* o = p + kHeader;
    for (int i = 0; i < q_limbs; i++, o += 8) put64(o, q[i]);
    const size_t words = (size_t)count * n * q_limbs;
    for (size_t i = 0; i < words; i++, o += 8) put64(o, polys[i]);
    put64(o, fnv1a(p, (size_t)(o - p)));
    return CY_OK;
}

cy_status cy_blob_info_read(const void* buf, size_t len, cy_blob_info* info) {
    if (!buf || !info) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    const unsigned char* p = static_cast<const unsigned char*>(buf);
    if (len < kHeader + 8) return set_error(CY_ERR_INVALID_ARGUMENT, "blob truncated");
    if (std::memcmp(p, kMagic, 4) != 0) return set_error(CY_ERR_INVALID_ARGUMENT, "not a cuyashe blob");
    if (get32(p + 4) != kVersion) return set_error(CY_ERR_UNSUPPORTED, "unknown blob version");
    std::memset(info, 0, sizeof(*info));
    info->kind = get32(p + 8);
    const uint32_t n = get32(p + 12), L = get32(p + 16), count = get32(p + 20);
    if (info->kind < CY_BLOB_CIPHERTEXTS || info->kind > CY_BLOB_KEYS || n < 1 || n > (1u << 20) || L < 1 ||
        L > CY_BLOB_MAX_LIMBS || count > (1u << 30))
        return set_error(CY_ERR_INVALID_ARGUMENT, "corrupt blob header");
    const size_t bytes = blob_bytes((int)n, (int)L, (int)count);
    if (len < bytes) return set_error(CY_ERR_INVALID_ARGUMENT, "blob truncated");
    if (fnv1a(p, bytes - 8) != get64(p + bytes - 8)) return set_error(CY_ERR_INVALID_ARGUMENT, "blob checksum mismatch");
    info->n = (int)n;
    info->q_limbs = (int)L;
    info->count = (int)count;
    info->t = get64(p + 24);
    info->w_bits = (int)get32(p + 32);
    for (uint32_t i = 0; i < L; i++) info->q[i] = get64(p + kHeader + 8 * i);
    info->bytes = bytes;
    return CY_OK;
}

cy_status cy_deserialize(const void* buf, size_t len, uint64_t* polys, size_t max_words) {
    cy_blob_info info;
    CY_TRY(cy_blob_info_read(buf, len, &info));
    const size_t words = (size_t)info.count * info.n * info.q_limbs;
    if (words > max_words || (words > 0 && !polys)) return set_error(CY_ERR_INVALID_ARGUMENT, "output too small");
    const unsigned char* o = static_cast<const unsigned char*>(buf) + kHeader + 8 * (size_t)info.q_limbs;
    for (size_t i = 0; i < words; i++, o += 8) polys[i] = get64(o);
    if (!coeffs_below_q(polys, (size_t)info.count * info.n, info.q, info.q_limbs))
        return set_error(CY_ERR_INVALID_ARGUMENT, "coefficient not in [0, q)");
    return CY_OK;
}

// Keys of a scheme: kind CY_BLOB_KEYS, polynomials f, h, evk_0 .. evk_{ell-1}.
cy_status cy_yashe_save_keys(const cy_yashe* y, void* buf, size_t len, size_t* needed) {
    if (!y) return set_error(CY_ERR_INVALID_ARGUMENT, "yashe handle is NULL");
    if (!y->has_keys) return set_error(CY_ERR_NO_KEYS, "no keys installed");
    const cy_ring* r = y->ring;
    std::vector<uint64_t> polys;
    if (buf) {
        polys.reserve(y->h_f.size() + y->h_h.size() + y->h_evk.size());
        polys.insert(polys.end(), y->h_f.begin(), y->h_f.end());
        polys.insert(polys.end(), y->h_h.begin(), y->h_h.end());
        polys.insert(polys.end(), y->h_evk.begin(), y->h_evk.end());
    }
    static const uint64_t dummy = 0;
    return cy_serialize(CY_BLOB_KEYS, r->n, r->q_limbs.data(), r->l64, y->t, y->w_bits,
                        buf ? polys.data() : &dummy, 2 + y->ell, buf, len, needed);
}

cy_status cy_yashe_load_keys(cy_yashe* y, const void* buf, size_t len) {
    if (!y) return set_error(CY_ERR_INVALID_ARGUMENT, "yashe handle is NULL");
    cy_blob_info info;
    CY_TRY(cy_blob_info_read(buf, len, &info));
    const cy_ring* r = y->ring;
    if (info.kind != CY_BLOB_KEYS) return set_error(CY_ERR_INVALID_ARGUMENT, "blob does not hold keys");
    bool same = info.n == r->n && info.q_limbs == r->l64 && info.t == y->t && info.w_bits == y->w_bits &&
                info.count == 2 + y->ell;
    for (int i = 0; same && i < r->l64; i++) same = info.q[i] == r->q_limbs[i];
    if (!same) return set_error(CY_ERR_INVALID_ARGUMENT, "keys were made for other parameters");
    std::vector<uint64_t> polys((size_t)info.count * info.n * info.q_limbs);
    CY_TRY(cy_deserialize(buf, len, polys.data(), polys.size()));
    const size_t poly = (size_t)r->n * r->l64;
    return cy_yashe_set_keys(y, polys.data(), polys.data() + poly, polys.data() + 2 * poly);
}

}  // extern "C"
