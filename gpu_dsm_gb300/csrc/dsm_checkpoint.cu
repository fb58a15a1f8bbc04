// Full-state checkpoint of an ensemble.  The reference's binary conformation
// file (common/ensemble.cu:342-354, chain.cu:236-250; dsm_save_file here)
// keeps only Z, Q, N and the CD rates: a run resumed from it restarts its
// clocks, random streams and G(t) accumulation.  This file adds what an exact
// resume needs:
//   - per chain: time in ticks, event counter (the Philox counter), event hash,
//     fixed-point scale, stall code, pending flow dt, next sample index, N_K,
//     MSD reference position (the ChainState records);
//   - the conformations in the reference layout (float4 {Qx,Qy,Qz,N} and CD
//     rates, z_max per chain);
//   - every correlator level: shift registers, FP64 lag sums, block averages,
//     counters;
//   - the ensemble's time and event totals.
// A versioned header records the shape (chains, z_max, N_K, flow/correlator
// kind, levels, p, m) and the random-stream identity (seed, stream, chain
// offset); loading checks all of them and a checksum of the payload before
// anything reaches the device, so a handle is never left half-restored by a
// bad file.  A run continued from the checkpoint gives the same bits as the
// run that wrote it.
#include <cstdint>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dsm.h"
#include "dsm_host.h"
#include "dsm_internal.h"

using dsm::ChainState;

namespace {

constexpr char kMagic[8] = {'D', 'S', 'M', 'C', 'K', 'P', 'T', '1'};
constexpr uint32_t kVersion = 1;

struct Header {
  char magic[8];
  uint32_t version, header_bytes;
  int64_t n_chains;
  int32_t cap, nk, flow, corr_kind, levels, corr_p, corr_m, chain_state_bytes;
  uint64_t seed;
  uint32_t stream, chain_offset;
  double t_done;
  uint64_t events_total;
  uint64_t payload_bytes;
  uint64_t checksum;
};

// 64-bit words, multiply-xor chain (FNV-style constants); the payload is a
// whole number of 8-byte words
uint64_t mix(uint64_t h, const void* p, size_t bytes) {
  const unsigned char* b = (const unsigned char*)p;
  size_t i = 0;
  for (; i + 8 <= bytes; i += 8) {
    uint64_t w;
    std::memcpy(&w, b + i, 8);
    h = (h ^ w) * 0x100000001B3ull;
  }
  for (; i < bytes; ++i) h = (h ^ b[i]) * 0x100000001B3ull;
  return h;
}

struct Part {
  void* dev;
  size_t bytes;
};

// device arrays of the checkpoint, in file order
std::vector<Part> parts(dsm_sim* s) {
  const size_t n = (size_t)s->P.n_chains, cap = (size_t)s->cap;
  std::vector<Part> v = {{s->d_cs, n * sizeof(ChainState)},
                         {s->d_QN, n * cap * sizeof(float4)},
                         {s->d_tau, n * cap * sizeof(float)}};
  if (s->corr) {
    const size_t L = (size_t)s->levels, p = (size_t)s->cp;
    v.push_back({s->d_cshift, n * L * p * 3 * sizeof(float)});
    v.push_back({s->d_cacc, n * L * p * sizeof(double)});
    v.push_back({s->d_cavg, n * L * 3 * sizeof(float)});
    v.push_back({s->d_ccnt, n * L * sizeof(int4)});
  }
  return v;
}

Header header_of(const dsm_sim* s) {
  Header h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.header_bytes = sizeof(Header);
  h.n_chains = s->P.n_chains;
  h.cap = s->cap;
  h.nk = s->P.nk;
  h.flow = s->flow ? 1 : 0;
  h.corr_kind = s->ck;
  h.levels = s->corr ? s->levels : 0;
  h.corr_p = s->corr ? s->cp : 0;
  h.corr_m = s->corr ? s->cm : 0;
  h.chain_state_bytes = (int32_t)sizeof(ChainState);
  h.seed = s->P.seed;
  h.stream = s->P.stream;
  h.chain_offset = s->P.chain_offset;
  h.t_done = s->t_done;
  h.events_total = s->events_total;
  return h;
}

int fail(dsm_sim* s, int code, const std::string& m) {
  s->err = m;
  return code;
}

}  // namespace

extern "C" int dsm_checkpoint_save(dsm_sim* s, const char* path) {
  const dsm::NvtxRange nvtx_range("dsm_checkpoint_save");
  if (!s || !s->ready || !path || s->pending) return DSM_ERR_INVALID;
  const std::vector<Part> ps = parts(s);
  Header h = header_of(s);
  std::vector<std::vector<unsigned char>> host(ps.size());
  uint64_t ck = 0xCBF29CE484222325ull;
  for (size_t i = 0; i < ps.size(); ++i) {
    host[i].resize(ps[i].bytes);
    const cudaError_t e = cudaMemcpyAsync(host[i].data(), ps[i].dev, ps[i].bytes, cudaMemcpyDeviceToHost, s->st);
    if (e != cudaSuccess) return fail(s, DSM_ERR_CUDA, std::string("checkpoint copy: ") + cudaGetErrorString(e));
  }
  const cudaError_t e = cudaStreamSynchronize(s->st);
  if (e != cudaSuccess) return fail(s, DSM_ERR_CUDA, std::string("checkpoint copy: ") + cudaGetErrorString(e));
  for (const auto& b : host) {
    ck = mix(ck, b.data(), b.size());
    h.payload_bytes += b.size();
  }
  h.checksum = ck;
  std::ofstream f(path, std::ios::binary);
  if (!f) return fail(s, DSM_ERR_INVALID, std::string("cannot open ") + path);
  f.write((const char*)&h, sizeof(h));
  for (const auto& b : host) f.write((const char*)b.data(), (std::streamsize)b.size());
  f.flush();
  return f ? DSM_OK : fail(s, DSM_ERR_INVALID, std::string("write failed: ") + path);
}

extern "C" int dsm_checkpoint_load(dsm_sim* s, const char* path) {
  const dsm::NvtxRange nvtx_range("dsm_checkpoint_load");
  if (!s || !s->ready || !path || s->pending) return DSM_ERR_INVALID;
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(s, DSM_ERR_INVALID, std::string("cannot open ") + path);
  Header h;
  f.read((char*)&h, sizeof(h));
  if (!f || std::memcmp(h.magic, kMagic, 8) != 0) return fail(s, DSM_ERR_INVALID, "not a checkpoint file");
  if (h.version != kVersion || h.header_bytes != sizeof(Header) || h.chain_state_bytes != (int32_t)sizeof(ChainState))
    return fail(s, DSM_ERR_INVALID, "checkpoint format version " + std::to_string(h.version) + " not supported");
  const Header me = header_of(s);
  auto differ = [&](const char* what) {
    return fail(s, DSM_ERR_INVALID, std::string("checkpoint does not match this ensemble: ") + what);
  };
  if (h.n_chains != me.n_chains) return differ("number of chains");
  if (h.cap != me.cap) return differ("z_max");
  if (h.nk != me.nk) return differ("N_K");
  if (h.flow != me.flow) return differ("flow / equilibrium");
  if (h.corr_kind != me.corr_kind || h.levels != me.levels || h.corr_p != me.corr_p || h.corr_m != me.corr_m)
    return differ("correlator (kind, levels, p, m)");
  if (h.seed != me.seed || h.stream != me.stream || h.chain_offset != me.chain_offset)
    return differ("random streams (seed, stream, chain offset)");
  const std::vector<Part> ps = parts(s);
  std::vector<std::vector<unsigned char>> host(ps.size());
  uint64_t ck = 0xCBF29CE484222325ull, total = 0;
  for (size_t i = 0; i < ps.size(); ++i) {
    host[i].resize(ps[i].bytes);
    f.read((char*)host[i].data(), (std::streamsize)ps[i].bytes);
    if (!f) return fail(s, DSM_ERR_INVALID, "truncated checkpoint file");
    ck = mix(ck, host[i].data(), ps[i].bytes);
    total += ps[i].bytes;
  }
  if (total != h.payload_bytes || ck != h.checksum) return fail(s, DSM_ERR_INVALID, "checkpoint checksum mismatch");
  // the chains' N_K must be this ensemble's (polydisperse ensembles keep them per chain)
  const ChainState* cs = (const ChainState*)host[0].data();
  for (int64_t i = 0; i < h.n_chains; ++i) {
    if (cs[i].nk != s->nk_chain[(size_t)i]) return differ("per-chain N_K");
    if (cs[i].Z < 1 || cs[i].Z > s->cap) return fail(s, DSM_ERR_INVALID, "corrupt checkpoint (Z out of range)");
  }
  for (size_t i = 0; i < ps.size(); ++i) {
    const cudaError_t e = cudaMemcpyAsync(ps[i].dev, host[i].data(), ps[i].bytes, cudaMemcpyHostToDevice, s->st);
    if (e != cudaSuccess) return fail(s, DSM_ERR_CUDA, std::string("restore copy: ") + cudaGetErrorString(e));
  }
  const cudaError_t e = cudaStreamSynchronize(s->st);
  if (e != cudaSuccess) return fail(s, DSM_ERR_CUDA, std::string("restore copy: ") + cudaGetErrorString(e));
  s->t_done = h.t_done;
  s->t_window = h.t_done;
  s->events_total = h.events_total;
  return DSM_OK;
}
