// Binary formats for device-resident keys and for ciphertexts (no counterpart in the reference, which has
// no serialisation): a server restarts with its keys reloaded by one host->device copy each, without
// regenerating or re-transforming them.
//
// Key record: a 96-byte header, then the key exactly as it sits in device memory (the NTT-domain form the
// key product reads: the wide form [limbs][pair][N/32][digits][2][32] of uint2 or the per-limb Montgomery
// form [limbs][digits][2][N]), limb-major, so a truncated Q-only key is the prefix of its limbs.
// Ciphertext record: a 64-byte header, then [components][level + 1][N] u64 residues (coefficient form).
// Both headers carry the ring degree and an FNV-1a fingerprint of the whole modulus chain (Q then P), which
// must match the loading context, and a checksum of the payload words.
#include <cstring>

#include "context.hpp"

using namespace rc;

namespace {

constexpr char KSK_MAGIC[8] = {'R', 'C', 'K', 'S', 'K', 'E', 'Y', '1'};
constexpr char CT_MAGIC[8] = {'R', 'C', 'C', 'T', 'X', 'T', '0', '1'};
constexpr uint32_t FORMAT_VERSION = 1;

struct KskHeader {
  char magic[8];
  uint32_t version, form;  // form: 0 per-limb Montgomery NTT, 1 wide (internal primes)
  uint64_t poly_degree;
  uint32_t digits;
  int32_t level;
  uint32_t aux, limbs;  // limbs stored
  uint64_t galois;
  uint64_t payload_bytes;
  uint64_t fingerprint;
  uint64_t checksum;
  uint64_t reserved[3];
};
static_assert(sizeof(KskHeader) == 96, "key header layout");

struct CtHeader {
  char magic[8];
  uint32_t version, components;
  uint64_t poly_degree;
  int32_t level, scale_bits;
  uint64_t payload_bytes;
  uint64_t fingerprint;
  uint64_t checksum;
  uint64_t reserved;
};
static_assert(sizeof(CtHeader) == 64, "ciphertext header layout");

uint64_t fnv1a(const void* p, size_t n, uint64_t h = 1469598103934665603ull) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t basis_fingerprint(const rc_context* c) {
  uint64_t h = fnv1a(&c->N, sizeof(c->N));
  for (uint64_t m : c->mod) h = fnv1a(&m, sizeof(m), h);
  return h;
}

// sum of the payload's 64-bit words with a rotating weight: detects truncation, reordering and flips
uint64_t payload_checksum(const uint64_t* w, size_t words) {
  uint64_t a = 0, b = 0;
  for (size_t i = 0; i < words; ++i) {
    a += w[i];
    b += a;
  }
  return a ^ (b << 1);
}

// bytes of `limbs` limbs of a resident key: the wide form holds two uint2 pairs per residue
size_t ksk_payload_bytes(size_t N, size_t limbs, size_t digits, bool wide) {
  return limbs * digits * 2 * N * 8 * (wide ? 2 : 1);
}

size_t ksk_payload_bytes(const rc_ksk* k) {
  return ksk_payload_bytes((size_t)k->ctx->N, k->limbs(), k->digits, k->wdata != nullptr);
}

}  // namespace

extern "C" int rc_ksk_serialized_size(const rc_ksk* k, uint64_t* bytes) {
  return guarded("rc_ksk_serialized_size", [&] {
    require(!k || !k->alpha, "RNS-hybrid keys are not serialisable");
    require(k && bytes, "arguments must not be null");
    *bytes = sizeof(KskHeader) + ksk_payload_bytes(k);
  });
}

extern "C" int rc_ksk_serialize(rc_context* c, const rc_ksk* k, void* host_buf, uint64_t buf_bytes, void* stream) {
  return guarded("rc_ksk_serialize", [&] {
    require(!k || !k->alpha, "RNS-hybrid keys are not serialisable");
    require(c && k && host_buf, "arguments must not be null");
    require(k->ctx == c, "keyswitch key belongs to another context");
    const size_t payload = ksk_payload_bytes(k);
    require(buf_bytes >= sizeof(KskHeader) + payload, "buffer too small for the serialized key");
    KskHeader h{};
    memcpy(h.magic, KSK_MAGIC, 8);
    h.version = FORMAT_VERSION;
    h.form = k->wdata ? 1 : 0;
    h.poly_degree = (uint64_t)c->N;
    h.digits = k->digits;
    h.level = k->level;
    h.aux = k->aux;
    h.limbs = k->limbs();
    h.galois = k->galois;
    h.payload_bytes = payload;
    h.fingerprint = basis_fingerprint(c);
    char* dst = (char*)host_buf;
    const void* src = k->wdata ? (const void*)k->wdata : (const void*)k->data;
    cuda_check(cudaMemcpyAsync(dst + sizeof(KskHeader), src, payload, cudaMemcpyDeviceToHost, (cudaStream_t)stream),
               "key download");
    cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "key download");
    h.checksum = payload_checksum((const uint64_t*)(dst + sizeof(KskHeader)), payload / 8);
    memcpy(dst, &h, sizeof(h));
  });
}

extern "C" int rc_ksk_deserialize(rc_context* c, const void* host_buf, uint64_t buf_bytes, rc_ksk** out) {
  return guarded("rc_ksk_deserialize", [&] {
    require(c && host_buf && out, "arguments must not be null");
    *out = nullptr;
    require(buf_bytes >= sizeof(KskHeader), "serialized key is truncated");
    KskHeader h;
    memcpy(&h, host_buf, sizeof(h));
    require(memcmp(h.magic, KSK_MAGIC, 8) == 0, "not a serialized keyswitch key");
    require(h.version == FORMAT_VERSION, "unsupported serialized key version");
    require(h.poly_degree == (uint64_t)c->N && h.fingerprint == basis_fingerprint(c),
            "serialized key was made for another modulus chain");
    require(h.level >= 0 && h.level < c->L, "keyswitch key level out of range for this context");
    require(h.aux == 0 || (int)h.aux == c->K, "eval-key context must match the keyswitch key auxiliary basis");
    require(h.digits >= 1 && h.limbs == (uint32_t)h.level + 1 + h.aux, "serialized key header is inconsistent");
    if (h.galois) context_galois_inverse(c, h.galois);
    const int Kk = h.aux ? c->K : 0;
    const int Dk = h.aux ? context_level(c, h.level + 1).digits : (int)h.digits;
    const bool wide = context_wide_applies(c, h.level + 1, Kk, Dk);
    require((h.form == 1) == wide, "serialized key form does not match this context");
    const size_t payload = ksk_payload_bytes((size_t)c->N, h.limbs, h.digits, wide);
    require(h.payload_bytes == payload && buf_bytes >= sizeof(KskHeader) + payload, "serialized key is truncated");
    const uint64_t* words = (const uint64_t*)((const char*)host_buf + sizeof(KskHeader));
    require(payload_checksum(words, payload / 8) == h.checksum, "serialized key checksum mismatch");
    std::shared_ptr<DevBuf> buf(new DevBuf(payload));
    cuda_check(cudaMemcpy(buf->p, words, payload, cudaMemcpyHostToDevice), "key upload");
    rc_ksk* k = new rc_ksk();
    k->ctx = c;
    if (wide) {
      k->wbuf = buf;
      k->wdata = (uint64_t*)buf->p;
    } else {
      k->buf = buf;
      k->data = (uint64_t*)buf->p;
    }
    k->digits = h.digits;
    k->level = h.level;
    k->aux = h.aux;
    k->galois = h.galois;
    *out = k;
  });
}

extern "C" int rc_ct_serialized_size(const rc_context* c, int32_t level, uint32_t components, uint64_t* bytes) {
  return guarded("rc_ct_serialized_size", [&] {
    require(c && bytes, "arguments must not be null");
    require(level >= 0 && level < c->L, "ciphertext level out of range for this context");
    require(components == 2 || components == 3, "a ciphertext has 2 or 3 components");
    *bytes = sizeof(CtHeader) + (uint64_t)components * (level + 1) * c->N * 8;
  });
}

extern "C" int rc_ct_serialize(rc_context* c, const rc_ciphertext* ct, uint32_t components, void* host_buf,
                               uint64_t buf_bytes, void* stream) {
  return guarded("rc_ct_serialize", [&] {
    require(c && host_buf, "arguments must not be null");
    context_check_ct(c, ct, "ciphertext");
    require(components == 2 || components == 3, "a ciphertext has 2 or 3 components");
    const size_t payload = (size_t)components * (ct->level + 1) * c->N * 8;
    require(buf_bytes >= sizeof(CtHeader) + payload, "buffer too small for the serialized ciphertext");
    char* dst = (char*)host_buf;
    cuda_check(cudaMemcpyAsync(dst + sizeof(CtHeader), ct->data, payload, cudaMemcpyDeviceToHost, (cudaStream_t)stream),
               "ciphertext download");
    cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "ciphertext download");
    CtHeader h{};
    memcpy(h.magic, CT_MAGIC, 8);
    h.version = FORMAT_VERSION;
    h.components = components;
    h.poly_degree = (uint64_t)c->N;
    h.level = ct->level;
    h.scale_bits = ct->scale_bits;
    h.payload_bytes = payload;
    h.fingerprint = basis_fingerprint(c);
    h.checksum = payload_checksum((const uint64_t*)(dst + sizeof(CtHeader)), payload / 8);
    memcpy(dst, &h, sizeof(h));
  });
}

extern "C" int rc_ct_header(const void* host_buf, uint64_t buf_bytes, uint64_t* poly_degree, int32_t* level,
                            int32_t* scale_bits, uint32_t* components) {
  return guarded("rc_ct_header", [&] {
    require(host_buf, "arguments must not be null");
    require(buf_bytes >= sizeof(CtHeader), "serialized ciphertext is truncated");
    CtHeader h;
    memcpy(&h, host_buf, sizeof(h));
    require(memcmp(h.magic, CT_MAGIC, 8) == 0, "not a serialized ciphertext");
    require(h.version == FORMAT_VERSION, "unsupported serialized ciphertext version");
    if (poly_degree) *poly_degree = h.poly_degree;
    if (level) *level = h.level;
    if (scale_bits) *scale_bits = h.scale_bits;
    if (components) *components = h.components;
  });
}

extern "C" int rc_ct_deserialize(rc_context* c, const void* host_buf, uint64_t buf_bytes, rc_ciphertext* out,
                                 uint64_t out_bytes, void* stream) {
  return guarded("rc_ct_deserialize", [&] {
    require(c && host_buf && out && out->data, "arguments must not be null");
    require(buf_bytes >= sizeof(CtHeader), "serialized ciphertext is truncated");
    CtHeader h;
    memcpy(&h, host_buf, sizeof(h));
    require(memcmp(h.magic, CT_MAGIC, 8) == 0, "not a serialized ciphertext");
    require(h.version == FORMAT_VERSION, "unsupported serialized ciphertext version");
    require(h.poly_degree == (uint64_t)c->N && h.fingerprint == basis_fingerprint(c),
            "serialized ciphertext was made for another modulus chain");
    require(h.level >= 0 && h.level < c->L, "ciphertext level out of range for this context");
    require(h.components == 2 || h.components == 3, "a ciphertext has 2 or 3 components");
    const size_t payload = (size_t)h.components * (h.level + 1) * c->N * 8;
    require(h.payload_bytes == payload && buf_bytes >= sizeof(CtHeader) + payload,
            "serialized ciphertext is truncated");
    // the record decides the size; a destination sized for a lower level must not be overrun
    require(out_bytes >= payload, "serialized ciphertext does not fit the destination buffer");
    const uint64_t* words = (const uint64_t*)((const char*)host_buf + sizeof(CtHeader));
    require(payload_checksum(words, payload / 8) == h.checksum, "serialized ciphertext checksum mismatch");
    cuda_check(cudaMemcpyAsync(out->data, words, payload, cudaMemcpyHostToDevice, (cudaStream_t)stream), "ciphertext upload");
    cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "ciphertext upload");
    out->level = h.level;
    out->scale_bits = h.scale_bits;
  });
}
