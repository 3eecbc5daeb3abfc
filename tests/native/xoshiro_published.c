/* Independent restatement of the published generators that the reference's
 * sampler uses, written from their published descriptions and not from the
 * oracle's code, so a CPU test can compare the two streams word for word.
 *
 *  - SplitMix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
 *    generators", OOPSLA 2014; the 64-bit variant with the mixing constants
 *    Vigna published beside xoshiro): the state advances by the golden-ratio
 *    increment 0x9e3779b97f4a7c15, and the output mixes it with xor-shifts by
 *    30, 27 and 31 and the multipliers 0xbf58476d1ce4e5b9, 0x94d049bb133111eb.
 *  - xoshiro256++ (Blackman and Vigna, "Scrambled linear pseudorandom number
 *    generators", ACM TOMS 2021): output rotl(s0 + s3, 23) + s0; then
 *    t = s1 << 17, s2 ^= s0, s3 ^= s1, s1 ^= s2, s0 ^= s3, s2 ^= t,
 *    s3 = rotl(s3, 45).
 *  - rand_xoshiro 0.7's seed_from_u64 (crates/pyre/src/sampler.rs:23 calls
 *    it): a SplitMix64 whose state starts at the seed fills the 32-byte seed
 *    with its outputs, little-endian, so state word k is its k-th output.
 *  - rand_xoshiro's next_u32: the upper 32 bits of next_u64.
 *  - rand 0.9's StandardUniform f32 (sampler.rs:30,34): the top 24 bits of a
 *    u32 times 2^-24.
 */
#include <stdint.h>

typedef struct { uint64_t s[4]; } pub_xoshiro;

static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t splitmix_next(uint64_t* x) {
    uint64_t z = (*x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static uint64_t xoshiro_next(pub_xoshiro* g) {
    uint64_t* s = g->s;
    const uint64_t result = rotl64(s[0] + s[3], 23) + s[0];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return result;
}

static void seed_from_u64(pub_xoshiro* g, uint64_t seed) {
    uint64_t x = seed;
    for (int k = 0; k < 4; ++k) g->s[k] = splitmix_next(&x);
}

/* n outputs of next_u64 after seed_from_u64(seed). */
void pub_u64_stream(uint64_t seed, uint32_t n, uint64_t* out) {
    pub_xoshiro g;
    seed_from_u64(&g, seed);
    for (uint32_t i = 0; i < n; ++i) out[i] = xoshiro_next(&g);
}

/* n f32 draws (rand's StandardUniform over next_u32) after seed_from_u64(seed). */
void pub_f32_stream(uint64_t seed, uint32_t n, float* out) {
    pub_xoshiro g;
    seed_from_u64(&g, seed);
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t u = (uint32_t)(xoshiro_next(&g) >> 32);
        out[i] = (float)(u >> 8) * (1.0f / 16777216.0f);
    }
}

/* n outputs of next_u64 from an explicit state (no seeding). */
void pub_u64_from_state(const uint64_t* state4, uint32_t n, uint64_t* out) {
    pub_xoshiro g;
    for (int k = 0; k < 4; ++k) g.s[k] = state4[k];
    for (uint32_t i = 0; i < n; ++i) out[i] = xoshiro_next(&g);
}

/* n outputs of SplitMix64 whose state starts at x0. */
void pub_splitmix_stream(uint64_t x0, uint32_t n, uint64_t* out) {
    uint64_t x = x0;
    for (uint32_t i = 0; i < n; ++i) out[i] = splitmix_next(&x);
}
