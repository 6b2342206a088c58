/*
 * mumfim_netgen.h -- seeded synthetic fiber networks for tests and benchmarks.
 *
 * The reference ships a few fixed networks (test/microscale/fiber_networks/)
 * and has no generator; this one produces networks of any size with the same
 * structure: nodes in the RVE cube [-0.5,0.5]^3, fibers = edges of the
 * undirected k-nearest-neighbour graph, nodes near a face snapped onto it so
 * that they become the fixed boundary of RVE.h:86-103.
 *
 * The generator uses only IEEE +,-,*,/ and integer arithmetic on a
 * std::mt19937_64 stream, so a (seed, n_nodes, k) triple gives the same
 * network on every platform.
 */
#ifndef MUMFIM_NETGEN_H
#define MUMFIM_NETGEN_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Generates one network.
 *  n_nodes  nodes drawn uniformly in [-0.5,0.5]^3 from mt19937_64(seed);
 *           each coordinate within `snap` of +-0.5 is set to +-0.5; a draw
 *           closer than `min_sep` to an earlier node is rejected and redrawn.
 *  k        neighbours per node; ties in distance go to the lower node id.
 *  coords   out, n_nodes x 3.
 *  conn     out, up to max_fibers x 2 (n_nodes * k always suffices); fibers
 *           are sorted by (lower id, higher id), duplicates removed.
 * Returns the number of fibers, or -1 on bad arguments / too small a buffer. */
int32_t mfg_generate_knn_network(int32_t n_nodes, int32_t k, uint64_t seed, double snap,
                                 double min_sep, double* coords, int32_t* conn,
                                 int32_t max_fibers);

/* Uniform double in [0,1) and a standard normal deviate (Marsaglia polar
 * method with a portable logarithm) from mt19937_64(seed), `n` values each,
 * for drawing per-RVE parameters reproducibly. */
void mfg_generate_uniform(uint64_t seed, int32_t n, double* out);
void mfg_generate_normal(uint64_t seed, int32_t n, double* out);
/* Portable exp and log built from +,-,*,/ only (used to turn normal deviates
 * into lognormal parameters identically on every platform). */
double mfg_portable_exp(double x);
double mfg_portable_log(double x);

#ifdef __cplusplus
}
#endif
#endif
