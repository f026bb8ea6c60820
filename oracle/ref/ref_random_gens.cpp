// Link-time replacement for the reference's src/random_gens.cpp
// (randomGen::RandomGens, include/LatticeDNAOrigami/random_gens.hpp:19-33).
// Every uniform_real()/uniform_int() call of the reference is served from one
// Philox stream instead of std::mt19937_64, so the reference, the oracle port
// and the CUDA engine consume identical random numbers in identical order.
#include "LatticeDNAOrigami/random_gens.hpp"
#include "philox_stream.h"

namespace {
ldo_ref::Stream g_stream;
}

extern "C" void ldo_ref_rng_configure(uint32_t seed, uint32_t replica, uint32_t stream) {
    g_stream.key[0] = seed;
    g_stream.key[1] = replica;
    g_stream.stream = stream;
    g_stream.draws = 0;
}

extern "C" uint64_t ldo_ref_rng_draws() { return g_stream.draws; }

namespace randomGen {

RandomGens::RandomGens() {}

RandomGens::~RandomGens() {}

void RandomGens::set_seed(int seed) {
    g_stream.key[0] = (uint32_t)seed;
    g_stream.draws = 0;
}

double RandomGens::uniform_real() { return g_stream.uniform_real(); }

int RandomGens::uniform_int(int lower, int upper) { return g_stream.uniform_int(lower, upper); }

} // namespace randomGen
