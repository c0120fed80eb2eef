// Device-resident continuous batching of independent CG systems (solve.cu):
// the iteration loop of the request server.  Plain C++ declarations, so the
// host-only server (serve.cpp) can drive it.
//
// A System is one request's CG, set up on any context: its preconditioner,
// initial residual, first z and rho — the first steps of llf_pcg, with the
// same kernels.  The Engine owns a table of slots in device memory (one per
// admitted system: its matrix and vectors) and a chunk table covering every
// admitted system, and replays one captured CUDA graph of 16 CG iterations
// over whatever the tables hold.  Systems are admitted and retired between
// replays, so a request that arrives while others iterate joins the next
// replay instead of waiting for the batch to drain.  Each system keeps its
// own chunks (768 DoFs from its first DoF), scalars and reductions in chunk
// order, so its iterates are those of a lone llf_pcg bit for bit.
#pragma once
#include <stdint.h>

#include <vector>

struct llf_ctx;
struct llf_matrix;

namespace llf_engine {

struct System;
struct Engine;

struct Done {
  int64_t tag = 0;
  int status = 0;          // LLF_OK, LLF_ERR_NOT_CONVERGED or LLF_ERR_NUMERIC
  int64_t iters = 0;
  double relres = 0.0;
  std::vector<double> x;   // the solution, fixed entries kept
};

// Set up the CG of K x = b (fixed entries of x0 prescribed; host arrays of
// K's DoF count) on ctx's stream, with a local preconditioner (none, Jacobi,
// block Jacobi).  Synchronises ctx's stream.  K must outlive the system.
int prepare(llf_ctx *ctx, const llf_matrix *K, const double *b, const double *x0, const uint8_t *fixed,
            int precond, double reltol, int64_t maxiter, System **out);
void release(llf_ctx *ctx, System *sys);

// An engine on ctx (its stream runs the iterations) for at most max_systems
// systems of at most max_chunks chunks (768 DoFs) in total.
int create(llf_ctx *ctx, int max_systems, int64_t max_chunks, Engine **out);
void destroy(Engine *e);

// Admit a prepared system under `tag`; 1 if admitted, 0 if no slot or chunk
// room is free (try again after a collect), < 0 on error.
int admit(Engine *e, System *sys, int64_t tag);
// Systems currently admitted.
int admitted(const Engine *e);
// One replay (16 iterations of every admitted system).
int step(Engine *e);
// Retire the systems that are done: their results are appended to out and
// their System objects are released on the engine's context.
int collect(Engine *e, std::vector<Done> &out);

}  // namespace llf_engine
