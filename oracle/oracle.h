/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C restatement of the reference's min-cut / connected-components hot path
 * (PJK/comm-avoiding-cuts-cc; single-threaded except orc_cc_iss_mt, which runs the per-rank
 * phases on host threads), used only to check the CUDA path:
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs may call
 * it; the product (libcac) never links or runs it.
 *
 * Pinning (see tests/test_oracle_pins.py):
 *   - sitmo block function: known-answer vectors dumped from the reference's own
 *     lib/prng_engine.hpp (tests/golden/sitmo_kat.txt);
 *   - connected components: labels and counts dumped from the reference's own
 *     UnweightedIteratedSparseSampling::connectedComponents (tests/golden/ref_test_inputs.json,
 *     cc_seeded.json);
 *   - exact minimum cut: values from the reference's test_inputs graph files and from its
 *     comincut::deterministic_minimum_cut on seeded graphs (tests/golden/ref_test_inputs.json,
 *     mincut_seeded.json);
 *   - approx_cut on the reference's own draws (orc_approx_cut_stream): libstdc++'s
 *     binomial_distribution on the reference engine (draws and engine position, from the
 *     binom_stream harness) and the answers of the reference's approx_cut executable on seeded
 *     graphs over 16 seeds each (tests/golden/approx_stream.json);
 *   - the per-trial replay of the counter-addressed square_root trial semantics has no reference
 *     counterpart (the reference's trial streams depend on libstdc++ distribution
 *     internals and on Boost's union-by-rank tie-breaks), so it is pinned at result
 *     level: every trial value is an upper bound on, and the minimum over trials equals,
 *     the exact Stoer-Wagner cut on the pinned graphs.
 */
#ifndef CAC_ORACLE_H
#define CAC_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- sitmo (lib/prng_engine.hpp:307-343 encrypt_counter, :195-212 operator()) ---- */
void orc_sitmo_block(const uint64_t key[4], const uint64_t ctr[4], uint64_t out[4]);
/* 32-bit output k of the reference engine sitmo::prng_engine(seed) (k-th call of operator()). */
uint32_t orc_sitmo_seed_output(uint32_t seed, uint64_t k);
/* Fill `count` consecutive 32-bit outputs of an engine whose key and counter were set with
 * set_key(key) / set_counter(ctr, 0) (lib/prng_engine.hpp:282-297). */
void orc_sitmo_outputs(const uint64_t key[4], const uint64_t ctr[4], uint64_t count, uint32_t *out);
/* u64 draw d of round `round` of stream `key`: word d&3 of the block at counter (d>>2, round, 0, 0). */
uint64_t orc_draw64(const uint64_t key[4], uint64_t round, uint64_t d);

/* ---- connected components ---- */
/* Canonical labels: label(v) = rank of min(component(v)) among all component minima, which is
 * what the reference's relabel-by-first-appearance produces (IteratedSparseSampling.hpp:210-220,
 * composed across rounds at UnweightedIteratedSparseSampling.cpp:60-62). Returns #components. */
uint32_t orc_cc_labels(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t *labels);
/* Restatement of the reference's iterated-sparse-sampling CC loop on `ranks` virtual ranks
 * (UnweightedIteratedSparseSampling.cpp:24-128, IteratedSparseSampling.hpp:160-295):
 * per round, every rank draws engine()%slice samples from its slice with sitmo(seed+rank),
 * the root shuffles, runs the prefix union-find to one component, relabels by first
 * appearance, and every rank rewrites its slice dropping loops. Writes labels (nullable),
 * returns #components; *rounds_out (nullable) receives the number of rounds. */
uint32_t orc_cc_iss(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t seed, uint32_t ranks,
                    uint32_t *labels, uint32_t *rounds_out);
/* the same with the per-rank phases on `threads` host threads (results identical) */
uint32_t orc_cc_iss_mt(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t seed, uint32_t ranks,
                       uint32_t threads, uint32_t *labels, uint32_t *rounds_out);
/* Sample count the reference asks for per round (UnweightedIteratedSparseSampling.cpp:82-85). */
uint64_t orc_cc_sample_count(uint32_t n, uint64_t edges_left);

/* ---- exact minimum cut ---- */
/* Stoer-Wagner on a dense symmetric n x n matrix (row-major, zero diagonal). The matrix is
 * consumed (modified). Returns UINT64_MAX for n < 2. */
uint64_t orc_stoer_wagner_dense(uint32_t n, uint64_t *mat);
/* Exact min cut of an edge list (builds the dense matrix; n <= ~10^4). */
uint64_t orc_exact_mincut(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w);
/* the same value by Nagamochi-Ono-Ibaraki contractions (fast on graphs of thousands of vertices) */
uint64_t orc_exact_mincut_noi(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w);

/* ---- square_root trial semantics ---- */
/* SquareRootCut::intermediate_size (SquareRootCut.cpp:63-70) with base_case_multiplier 2. */
uint32_t orc_intermediate_size(uint32_t n, uint64_t m);
/* SquareRootCut::numberOfTrials (SquareRootCut.cpp:76-83). */
uint32_t orc_number_of_trials(uint32_t n, uint64_t m, double success_probability);
/* comincut::min_success_in_one_trial (co_mincut.cpp:32-41). */
double orc_min_success_in_one_trial(int n);
/* comincut::target_number_of_vertices_for_contraction (co_mincut.cpp:18-20). */
int orc_ks_target(int n);
/* One counter-addressed square_root trial (virtual rank r, trial index i); returns its cut. */
uint64_t orc_mincut_trial(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                          uint32_t seed, uint32_t rank, uint32_t trial);
/* Only the Karger-Stein part (Stage 3) on a dense matrix, for kernel-level parity. */
uint64_t orc_ks_dense(uint32_t n, const uint64_t *mat, uint32_t seed, uint32_t rank, uint32_t trial);
/* one plain Karger-Stein trial (dense or sparse root) and the dense-node limit of both */
uint64_t orc_ks_trial(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w, uint32_t seed,
                      uint32_t trial);
void orc_set_dense_limit(uint32_t n);
/* the high-concurrency group variant: trial count for (ranks, trials) and one group's trial */
uint32_t orc_group_count(uint32_t ranks, uint32_t trials);
uint32_t orc_group_draws(uint32_t n);
uint64_t orc_mincut_group_trial(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                                uint32_t seed, uint32_t group);
/* Only Stage 1+2: contract to t vertices and emit the dense t' x t' matrix (returns t';
 * `mat_out` must hold n*n entries or NULL to only return t'). */
uint32_t orc_shrink_to_dense(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                             uint32_t target, uint32_t seed, uint32_t rank, uint32_t trial, uint64_t *mat_out);
/* Full square_root run: min over ranks*ceil(T/ranks) trials. trials_per_rank_out nullable. */
uint64_t orc_square_root(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                         double success_probability, uint32_t seed, uint32_t ranks, uint32_t *trials_per_rank_out);

/* ---- approx_cut ---- */
uint32_t orc_approx_trials(double success_probability);
/* Fixed-point (1 - 2^-level)^w as a 0.64 fraction (w >= 1, 1 <= level <= 63). */
uint64_t orc_keep_threshold(uint32_t level, uint32_t w);
/* Returns the cut estimate 2^level; *levels_out (nullable) = first disconnected level. */
uint64_t orc_approx_cut(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                        double success_probability, uint32_t seed, uint32_t ranks, uint32_t *levels_out);
/* The same run on the reference's own draws (libstdc++ binomial_distribution on
 * sitmo::prng_engine(seed + r)); returns 0 where a draw leaves the restated regime
 * (weight * 2^-level >= 8). */
uint64_t orc_approx_cut_stream(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                               double success_probability, uint32_t seed, uint32_t ranks, uint32_t *levels_out);
/* `count` consecutive draws binomial_distribution<int>(w[k % nw], 2^-level) on
 * sitmo::prng_engine(seed), then the engine's next raw output; -1 outside the restated regime. */
int orc_ref_binomial_draws(uint32_t seed, uint32_t level, uint64_t count, const uint32_t *w, uint32_t nw,
                           int32_t *draws, uint32_t *next_output);

#ifdef __cplusplus
}
#endif

#endif
