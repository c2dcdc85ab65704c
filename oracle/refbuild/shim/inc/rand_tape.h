// Control of the draw tape kept by oracle/refbuild/Rand_tape.cpp (test
// infrastructure). The reference's Rand (star-polymers/lib/Rand.h:10-29) is a
// process-global mt19937_64 seeded with 1 plus libstdc++ distributions; the
// tape records every value it hands out, in order, with the kind of draw, so
// the per-cell random numbers of an MPC collision can be handed to another
// implementation on identical inputs.
#ifndef SMPC_ORACLE_RAND_TAPE_H
#define SMPC_ORACLE_RAND_TAPE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { TAPE_UNIFORM = 1, TAPE_GAMMA = 2, TAPE_NORMAL = 3, TAPE_CHISQ = 4 };

void rand_tape_enable(int on);
void rand_tape_clear(void);
long rand_tape_size(void);
// Copies the first n entries (value, kind) out of the tape.
void rand_tape_copy(double* values, int* kinds, long n);
// Re-seeds the global engine and resets every distribution's internal state.
void rand_tape_reseed(unsigned long long seed);

#ifdef __cplusplus
}
#endif
#endif
