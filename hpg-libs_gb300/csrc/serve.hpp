// serve.hpp -- the serving form (serve.cu): a request loop with continuous
// batching over the graph-replayed batched pipeline.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include "engine.hpp"
#include "hpg_bwt_records.h"

namespace hpgbwt {

struct Server;

// The server takes over the engine's stream until destroyed.  hbm_budget 0:
// a quarter of the device memory free at creation.
Server* server_create(Engine* e, size_t max_batch_reads, uint64_t max_batch_bases, uint64_t hbm_budget,
                      uint32_t max_results, std::string* err);
void server_destroy(Server* s);  // finishes every queued request first
// The reads stay in the caller's memory until server_wait returns for the ticket.
int server_submit(Server* s, const char* seqs, const uint64_t* offs, size_t n, uint64_t* ticket, std::string* err);
// 0 done (view filled; valid until server_release), 1 timed out, -1 failed.
int server_wait(Server* s, uint64_t ticket, hpg_result_set_t* view, double* latency_ms, int timeout_ms,
                std::string* err);
int server_release(Server* s, uint64_t ticket, std::string* err);
void server_stats(Server* s, double* out, int n);

}  // namespace hpgbwt
