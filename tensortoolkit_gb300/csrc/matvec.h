// The two-site effective-Hamiltonian matvec object (matvec.cu), shared with the Lanczos
// driver (lanczos.cu).
#pragma once

#include <vector>

#include "ctrct.h"

namespace qltg {
}

using qltg::CtrctPlan;
using qltg::DevBuf;

struct qltg_matvec {
  qltg_ctx* ctx = nullptr;
  int mode = QLTG_MODE_FP64;
  CtrctPlan step[4];
  DevBuf t[3];
  const void* lenv = nullptr;
  const void* mpo1 = nullptr;
  const void* mpo2 = nullptr;
  const void* renv = nullptr;
  int64_t psi_size = 0;
  DevBuf psi_stage, out_stage;   // device copies of host psi / result (qltg_matvec_apply_host)
  struct Graph {
    const void* in;
    void* out;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
  };
  std::vector<Graph> graphs;
  cudaStream_t capture_stream = nullptr;

  ~qltg_matvec() {
    for (auto& g : graphs) {
      cudaGraphExecDestroy(g.exec);
      cudaGraphDestroy(g.graph);
    }
    if (capture_stream) cudaStreamDestroy(capture_stream);
  }

  bool fused_fields = false;   // split mode: the MPO step writing t3 folds the row scales of step 3's A

  // The two MPO steps as one contraction, t3 = t1 . W12, with W12 = W1 . W2 contracted over
  // the middle MPO bond once at creation (a constant of w d^2 d^2 w elements). Same result
  // (to rounding); it skips writing and reading t2 and, where the bond is small, does fewer
  // multiply-adds. Chosen at creation when it times faster than the two steps.
  bool mpo_fusable = false, mpo_fused = false;
  bool frozen = false;         // a Lanczos captured this matvec: its form no longer changes
  CtrctPlan mpo12;
  DevBuf w12;
  float mid_ms[2] = {0.f, 0.f};   // the MPO part timed at creation: two steps, fused
  CtrctPlan& mpo_producer() { return mpo_fused ? mpo12 : step[2]; }

  void enqueue_mid(cudaStream_t s) {
    if (fused_fields)
      QLTG_CUDA(cudaMemsetAsync(step[3].split->a_exps.get(), 0, step[3].split->n_a_rows * sizeof(int32_t), s));
    if (mpo_fused) {
      qltg::exec_contraction(mpo12, t[0].get(), w12.get(), t[2].get(), mode, s);
    } else {
      qltg::exec_contraction(step[1], t[0].get(), mpo1, t[1].get(), mode, s);
      qltg::exec_contraction(step[2], t[1].get(), mpo2, t[2].get(), mode, s);
    }
  }

  void enqueue(const void* psi, void* out, cudaStream_t s) {
    qltg::exec_contraction(step[0], lenv, psi, t[0].get(), mode, s);
    enqueue_mid(s);
    qltg::exec_contraction(step[3], t[2].get(), renv, out, mode, s);
  }

  cudaGraphExec_t graph_for(const void* in, void* out) {
    for (auto& g : graphs)
      if (g.in == in && g.out == out) return g.exec;
    if (graphs.size() >= 8) {
      cudaGraphExecDestroy(graphs.front().exec);
      cudaGraphDestroy(graphs.front().graph);
      graphs.erase(graphs.begin());
    }
    Graph g{in, out, nullptr, nullptr};
    QLTG_CUDA(cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue(in, out, capture_stream);
    } catch (...) {
      cudaGraph_t junk;
      cudaStreamEndCapture(capture_stream, &junk);
      if (junk) cudaGraphDestroy(junk);
      throw;
    }
    QLTG_CUDA(cudaStreamEndCapture(capture_stream, &g.graph));
    QLTG_CUDA(cudaGraphInstantiate(&g.exec, g.graph, 0));
    graphs.push_back(g);
    return g.exec;
  }
};

