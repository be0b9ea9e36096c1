// batch_solve.cu -- many root solves of uneven plasmas in one device-resident
// loop (alps_solve_many).
//
// The reference polishes one root at a time: every secant iteration is one
// disp() call, an MPI collective (src/ALPS_fns.f90:1919-2101).  Here n roots,
// each on its own context (its own plasma and k: grids, species and nmax
// differ from root to root), advance together on the device:
//
//   * each root owns two frequency slots; the root-finder state machines of
//     root_machine.cuh live in device memory (one RootState per root);
//   * one round is the fused det D launch over every root's slots (the four
//     kernels of launch_disp_multi, each root's context with the launch shape
//     of a lone batch of two, so its determinants do not depend on the
//     others) followed by k_root_step, which feeds each root its
//     determinants and writes the frequencies it asks for next;
//   * the rounds repeat inside one CUDA graph through a conditional WHILE
//     node: k_root_cond clears the condition once no root is active (or after
//     a bounded number of rounds), so the host neither waits for nor
//     launches any round.  One graph launch solves the whole batch.
//
// Each root's job keeps the launch shape of a batch of two, but its
// frequency count in the device job table follows the root: two, one (most
// secant iterations ask for one determinant) or none once the root is done,
// so the kernels evaluate only what the machines asked for.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "alps_internal.cuh"
#include "root_machine.cuh"

namespace {

// the frequency count of root r's job in the device job table: the
// kernels evaluate only that many of its two slots (none once it is done)
__device__ __forceinline__ void set_job_n(unsigned char* jobs, size_t stride, size_t noff, int r, int n) {
  *reinterpret_cast<int*>(jobs + (size_t)r * stride + noff) = n;
}

__global__ void k_root_init(const RootState* __restrict__ st, int n, unsigned char* jobs, size_t stride,
                            size_t noff) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) set_job_n(jobs, stride, noff, r, st[r].nwant);
}

__global__ void k_root_step(RootState* __restrict__ st, const RootParams* __restrict__ pr, double2* __restrict__ om,
                            const double2* __restrict__ D, int n, int* active, unsigned char* jobs, size_t stride,
                            size_t noff) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  RootState s = st[r];
  if (s.nwant > 0) {
    const double2 got[2] = {D[2 * r], D[2 * r + 1]};
    root_feed(s, pr[r], got);
    st[r] = s;
  }
  if (s.nwant > 0) {
    atomicAdd(active, 1);
    om[2 * r] = s.want[0];
    om[2 * r + 1] = (s.nwant > 1) ? s.want[1] : s.want[0];
  }
  set_job_n(jobs, stride, noff, r, s.nwant);
}

// one thread: ends the loop when no root is active or the round limit is hit
__global__ void k_root_cond(int* active, int* rounds, int max_rounds, cudaGraphConditionalHandle h) {
  const int a = *active;
  *active = 0;
  const int r = ++*rounds;
  if (a == 0 || r >= max_rounds) cudaGraphSetConditional(h, 0);
}

}  // namespace

extern "C" int alps_solve_many(alps_ctx* const* ctx, int n, int method, alps_complex* om, double om_rtol,
                               int* iters, alps_complex* Dfinal, int* converged) {
  if (n < 0 || (n > 0 && (!ctx || !om))) return ALPS_E_INVALID;
  if (method < 0 || method > 2 || !(om_rtol >= 0.0)) return ALPS_E_INVALID;
  if (n == 0) return ALPS_OK;
  int numiter_max = 1;
  for (int r = 0; r < n; ++r) {
    const alps_ctx* c = ctx[r];
    if (!c || !c->kset) return ALPS_E_INVALID;
    if (!ctx_fusable(c)) return ALPS_E_UNSUPPORTED;  // relativistic and closed-form species run per context
    numiter_max = std::max(numiter_max, c->sys.numiter);
  }
  // host side: the root machines' first requests
  std::vector<RootState> hs(n);
  std::vector<RootParams> hp(n);
  std::vector<double2> hom(2 * (size_t)n);
  for (int r = 0; r < n; ++r) {
    hp[r] = root_params(ctx[r]->sys, om_rtol);
    root_start(hs[r], hp[r], method, make_double2(om[r].re, om[r].im));
    hom[2 * r] = hs[r].want[0];
    hom[2 * r + 1] = hs[r].nwant > 1 ? hs[r].want[1] : hs[r].want[0];
  }
  cudaStream_t st = nullptr;
  ALPS_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  RootState* d_st = nullptr;
  RootParams* d_pr = nullptr;
  double2 *d_om = nullptr, *d_D = nullptr;
  int *d_flags = nullptr, *d_ctl = nullptr;
  MultiScratch* scratch = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int status = ALPS_OK;
  auto fail = [&](int code) {
    if (!status) status = code;
  };
  std::vector<int> nslot(n, 2);
  MultiLaunch ml;
  const int max_rounds = 3 * numiter_max + 16;  // every machine finishes within 2 numiter + 4 rounds
  do {
    if (cudaMalloc(&d_st, sizeof(RootState) * n) != cudaSuccess || cudaMalloc(&d_pr, sizeof(RootParams) * n) !=
                                                                        cudaSuccess ||
        cudaMalloc(&d_om, sizeof(double2) * 2 * n) != cudaSuccess ||
        cudaMalloc(&d_D, sizeof(double2) * 2 * n) != cudaSuccess || cudaMalloc(&d_flags, sizeof(int) * n) !=
                                                                         cudaSuccess ||
        cudaMalloc(&d_ctl, 2 * sizeof(int)) != cudaSuccess) {
      fail(ALPS_E_OOM);
      break;
    }
    if (cudaMemcpyAsync(d_st, hs.data(), sizeof(RootState) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(d_pr, hp.data(), sizeof(RootParams) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(d_om, hom.data(), sizeof(double2) * 2 * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(d_ctl, 0, 2 * sizeof(int), st) != cudaSuccess) {
      fail(ALPS_E_CUDA);
      break;
    }
    // job table and scratch of the fused rounds, built once
    int rc = prepare_disp_multi(ctx, nslot.data(), n, d_om, d_D, d_flags, &scratch, st, &ml);
    if (rc) {
      fail(rc);
      break;
    }
    // each job evaluates only the frequencies its root asks for
    size_t jstride = 0, jnoff = 0;
    disp_job_layout(&jstride, &jnoff);
    unsigned char* djobs = const_cast<unsigned char*>(static_cast<const unsigned char*>(ml.jobs));
    k_root_init<<<(n + 127) / 128, 128, 0, st>>>(d_st, n, djobs, jstride, jnoff);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
      fail(ALPS_E_CUDA);
      break;
    }
    // graph: WHILE (condition) { fused det D; root step; condition }
    cudaGraphConditionalHandle cond;
    if (cudaGraphCreate(&graph, 0) != cudaSuccess ||
        cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
      fail(ALPS_E_CUDA);
      break;
    }
    alignas(cudaGraphNodeParams) unsigned char cp_raw[sizeof(cudaGraphNodeParams)];
    memset(cp_raw, 0, sizeof(cp_raw));
    cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cp_raw);
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp) != cudaSuccess) {
      fail(ALPS_E_CUDA);
      break;
    }
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if (cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
        cudaSuccess) {
      fail(ALPS_E_CUDA);
      break;
    }
    rc = run_disp_multi(ml, st);
    if (!rc) {
      k_root_step<<<(n + 127) / 128, 128, 0, st>>>(d_st, d_pr, d_om, d_D, n, d_ctl, djobs, jstride, jnoff);
      k_root_cond<<<1, 1, 0, st>>>(d_ctl, d_ctl + 1, max_rounds, cond);
      if (cudaGetLastError() != cudaSuccess) rc = ALPS_E_CUDA;
    }
    cudaGraph_t captured = nullptr;
    if (cudaStreamEndCapture(st, &captured) != cudaSuccess && !rc) rc = ALPS_E_CUDA;
    if (rc) {
      fail(rc);
      break;
    }
    if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
      fail(ALPS_E_CUDA);
      break;
    }
    if (cudaGraphLaunch(exec, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
      fail(ALPS_E_CUDA);
      break;
    }
    if (cudaMemcpy(hs.data(), d_st, sizeof(RootState) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
      fail(ALPS_E_CUDA);
      break;
    }
    std::vector<int> fl(n);
    if (cudaMemcpy(fl.data(), d_flags, sizeof(int) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
      fail(ALPS_E_CUDA);
      break;
    }
    for (int r = 0; r < n; ++r)
      if (fl[r]) fail(ALPS_E_INVALID);  // resonant-order slots overflowed in some round
  } while (false);
  if (!status)
    for (int r = 0; r < n; ++r) {
      om[r] = alps_complex{hs[r].om.x, hs[r].om.y};
      if (iters) iters[r] = hs[r].iter;
      if (Dfinal) Dfinal[r] = alps_complex{hs[r].Dfin.x, hs[r].Dfin.y};
      if (converged) converged[r] = (hs[r].nwant == 0 && hs[r].converged) ? 1 : 0;
    }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  multi_scratch_free(scratch);
  cudaFree(d_st);
  cudaFree(d_pr);
  cudaFree(d_om);
  cudaFree(d_D);
  cudaFree(d_flags);
  cudaFree(d_ctl);
  cudaStreamDestroy(st);
  return status;
}
