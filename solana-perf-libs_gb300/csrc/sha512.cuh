// SHA-512 (FIPS 180-4) for the Ed25519 challenge H(R || A || M) and the
// signing nonce H(prefix || M), read straight from the packet buffer.
//
// Replaces the reference's LibTomCrypt SHA-512 (src/cuda-ecc-ed25519/
// sha512.cu: sha512_compress :96, sha512_update, sha512_final).  The
// message is never copied: each 64-bit big-endian schedule word is
// assembled from aligned 32-bit loads of the (up to three) byte ranges the
// hash covers, padding and the bit length are synthesised in registers.
#pragma once
#include <stdint.h>

static __constant__ uint64_t kSha512K[80] = {
    0x428a2f98d728ae22ULL, 0x7137449123ef65cdULL, 0xb5c0fbcfec4d3b2fULL, 0xe9b5dba58189dbbcULL,
    0x3956c25bf348b538ULL, 0x59f111f1b605d019ULL, 0x923f82a4af194f9bULL, 0xab1c5ed5da6d8118ULL,
    0xd807aa98a3030242ULL, 0x12835b0145706fbeULL, 0x243185be4ee4b28cULL, 0x550c7dc3d5ffb4e2ULL,
    0x72be5d74f27b896fULL, 0x80deb1fe3b1696b1ULL, 0x9bdc06a725c71235ULL, 0xc19bf174cf692694ULL,
    0xe49b69c19ef14ad2ULL, 0xefbe4786384f25e3ULL, 0x0fc19dc68b8cd5b5ULL, 0x240ca1cc77ac9c65ULL,
    0x2de92c6f592b0275ULL, 0x4a7484aa6ea6e483ULL, 0x5cb0a9dcbd41fbd4ULL, 0x76f988da831153b5ULL,
    0x983e5152ee66dfabULL, 0xa831c66d2db43210ULL, 0xb00327c898fb213fULL, 0xbf597fc7beef0ee4ULL,
    0xc6e00bf33da88fc2ULL, 0xd5a79147930aa725ULL, 0x06ca6351e003826fULL, 0x142929670a0e6e70ULL,
    0x27b70a8546d22ffcULL, 0x2e1b21385c26c926ULL, 0x4d2c6dfc5ac42aedULL, 0x53380d139d95b3dfULL,
    0x650a73548baf63deULL, 0x766a0abb3c77b2a8ULL, 0x81c2c92e47edaee6ULL, 0x92722c851482353bULL,
    0xa2bfe8a14cf10364ULL, 0xa81a664bbc423001ULL, 0xc24b8b70d0f89791ULL, 0xc76c51a30654be30ULL,
    0xd192e819d6ef5218ULL, 0xd69906245565a910ULL, 0xf40e35855771202aULL, 0x106aa07032bbd1b8ULL,
    0x19a4c116b8d2d0c8ULL, 0x1e376c085141ab53ULL, 0x2748774cdf8eeb99ULL, 0x34b0bcb5e19b48a8ULL,
    0x391c0cb3c5c95a63ULL, 0x4ed8aa4ae3418acbULL, 0x5b9cca4f7763e373ULL, 0x682e6ff3d6b2b8a3ULL,
    0x748f82ee5defb2fcULL, 0x78a5636f43172f60ULL, 0x84c87814a1f0ab72ULL, 0x8cc702081a6439ecULL,
    0x90befffa23631e28ULL, 0xa4506cebde82bde9ULL, 0xbef9a3f7b2c67915ULL, 0xc67178f2e372532bULL,
    0xca273eceea26619cULL, 0xd186b8c721c0c207ULL, 0xeada7dd6cde0eb1eULL, 0xf57d4f7fee6ed178ULL,
    0x06f067aa72176fbaULL, 0x0a637dc5a2c898a6ULL, 0x113f9804bef90daeULL, 0x1b710b35131c471bULL,
    0x28db77f523047d84ULL, 0x32caab7b40c72493ULL, 0x3c9ebe0a15c9bebcULL, 0x431d67c49c100d4cULL,
    0x4cc5d4becb3e42b6ULL, 0x597f299cfc657e2aULL, 0x5fcb6fab3ad6faecULL, 0x6c44198c4a475817ULL};

__device__ __forceinline__ uint64_t rotr64(uint64_t x, int n) { return (x >> n) | (x << (64 - n)); }

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

// 4 bytes at an arbitrary byte offset of a buffer of len bytes (base 4-byte
// aligned), little-endian, from at most two aligned 32-bit loads.  An
// aligned word is only read when it starts inside the buffer, so nothing
// past the last aligned word holding a buffer byte is ever touched; bytes
// at or past len come back as whatever that word holds (or zero).
__device__ __forceinline__ uint32_t ld_u32_any(const uint8_t* base, uint64_t off, uint64_t len) {
    const uint64_t a = off & ~3ull;
    const uint32_t sh = (uint32_t)(off & 3u) * 8u;
    const uint32_t* w = reinterpret_cast<const uint32_t*>(base + a);
    uint32_t lo = (a < len) ? __ldg(w) : 0u;
    uint32_t hi = (sh != 0u && a + 4 < len) ? __ldg(w + 1) : 0u;
    return __funnelshift_r(lo, hi, sh);
}

// 8 bytes at base+off as a big-endian 64-bit word.
__device__ __forceinline__ uint64_t ld_be64_any(const uint8_t* base, uint64_t off, uint64_t len) {
    uint32_t a = ld_u32_any(base, off, len);
    uint32_t b = ld_u32_any(base, off + 4, len);
    return ((uint64_t)bswap32(a) << 32) | bswap32(b);
}

// Message word q..q+8 of a message of length m at base+moff, with the
// SHA padding byte 0x80 at index m and zeros after it.
__device__ __forceinline__ uint64_t sha512_msg_word(const uint8_t* base, uint64_t len, uint64_t moff, uint32_t m,
                                                    uint32_t q) {
    if (q + 8 <= m) return ld_be64_any(base, moff + q, len);
    uint64_t w = 0;
    if (q < m) {
        uint32_t keep = m - q;  // 1..7 bytes
        w = ld_be64_any(base, moff + q, len) & (~0ull << (64 - 8 * keep));
    }
    if (q <= m && m < q + 8) w |= 0x80ull << (56 - 8 * (m - q));
    return w;
}

__device__ __forceinline__ void sha512_compress(uint64_t st[8], uint64_t W[16]) {
    uint64_t a = st[0], b = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6], h = st[7];
#pragma unroll
    for (int t = 0; t < 80; t++) {
        uint64_t w;
        if (t < 16) {
            w = W[t];
        } else {
            uint64_t w15 = W[(t - 15) & 15], w2 = W[(t - 2) & 15];
            uint64_t s0 = rotr64(w15, 1) ^ rotr64(w15, 8) ^ (w15 >> 7);
            uint64_t s1 = rotr64(w2, 19) ^ rotr64(w2, 61) ^ (w2 >> 6);
            w = W[t & 15] + s0 + W[(t - 7) & 15] + s1;
            W[t & 15] = w;
        }
        uint64_t t1 = h + (rotr64(e, 14) ^ rotr64(e, 18) ^ rotr64(e, 41)) + ((e & f) ^ (~e & g)) + kSha512K[t] + w;
        uint64_t t2 = (rotr64(a, 28) ^ rotr64(a, 34) ^ rotr64(a, 39)) + ((a & b) ^ (a & c) ^ (b & c));
        h = g;
        g = f;
        f = e;
        e = d + t1;
        d = c;
        c = b;
        b = a;
        a = t1 + t2;
    }
    st[0] += a; st[1] += b; st[2] += c; st[3] += d;
    st[4] += e; st[5] += f; st[6] += g; st[7] += h;
}

__device__ __forceinline__ void sha512_init(uint64_t st[8]) {
    st[0] = 0x6a09e667f3bcc908ULL; st[1] = 0xbb67ae8584caa73bULL;
    st[2] = 0x3c6ef372fe94f82bULL; st[3] = 0xa54ff53a5f1d36f1ULL;
    st[4] = 0x510e527fade682d1ULL; st[5] = 0x9b05688c2b3e6c1fULL;
    st[6] = 0x1f83d9abfb41bd6bULL; st[7] = 0x5be0cd19137e2179ULL;
}

// SHA-512 over  npre big-endian 64-bit words held in registers (npre <= 8,
// the prefix always lies inside the first block) || m message bytes at
// base+moff.  Ed25519 uses it as H(R || A || M) (npre = 8) for the verify
// and signing challenges and as H(prefix || M) (npre = 4) for the signing
// nonce.  The digest is returned as the 512-bit little-endian integer that
// the reference's sc_reduce reads (sc.cu:238), in sixteen 32-bit words.
static __device__ __noinline__ void sha512_prefixed(uint32_t out[16], const uint64_t pre[], int npre,
                                             const uint8_t* base, uint64_t len, uint64_t moff, uint32_t m) {
    uint64_t st[8];
    sha512_init(st);
    const uint32_t total = (uint32_t)npre * 8u + m;             // bytes hashed
    const uint32_t nblocks = (total + 17u + 127u) / 128u;
    const uint64_t bits = (uint64_t)total * 8ull;
#pragma unroll 1
    for (uint32_t blk = 0; blk < nblocks; blk++) {
        uint64_t W[16];
#pragma unroll
        for (int k = 0; k < 16; k++) {
            uint64_t w;
            if (blk == 0 && k < npre) {
                w = pre[k];
            } else {
                uint32_t pos = blk * 128u + 8u * (uint32_t)k;   // stream offset of this word
                w = sha512_msg_word(base, len, moff, m, pos - (uint32_t)npre * 8u);
            }
            if (blk == nblocks - 1) {
                if (k == 14) w = 0;
                if (k == 15) w = bits;
            }
            W[k] = w;
        }
        sha512_compress(st, W);
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        out[2 * i] = bswap32((uint32_t)(st[i] >> 32));
        out[2 * i + 1] = bswap32((uint32_t)st[i]);
    }
}
