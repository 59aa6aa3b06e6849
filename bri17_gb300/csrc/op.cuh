// op.cuh -- the operator handle shared by the library's translation units.
#pragma once

#include "common.cuh"
#include "df64.cuh"

namespace bri17gb {
struct CgState;
}

struct bri17_op {
  bri17gb::Geometry g;
  double L[3];
  double mu;
  double nu;
  int precision;  // bri17_precision
  int device;
  double cell_volume;  // |h|, accumulated like tests/test_bri17.cpp:93-97
  double corr;         // |h| / |N|, tests/test_bri17.cpp:98

  void* table_mem;                 // one device allocation for all tables
  bri17gb::Tables<double> tab64;   // always present (per-mode batch API)
  bri17gb::Tables<float> tab32;    // F32 handles only

  void* spec;          // half spectrum, spec_comps * g.cspec complex
  int spec_comps;
  void* stage_in;      // host-API staging buffers (lazy)
  void* stage_out;
  size_t stage_bytes;
  cudaStream_t copy_stream;   // host-API copies (lazy)
  cudaEvent_t host_events[64]; // host-API pipeline events (lazy, reused)

  // Conjugate-gradient work space (lazy, owned by cg.cu).
  void* cg_work;
  void (*cg_free)(void*);
  bri17_op* twin32;    // FP32 twin of an FP64 handle for mixed-precision CG
  unsigned material_epoch;  // bumped by bri17_op_set_material
  void* timing;             // PassTiming while per-pass timing is enabled
  int fused_form;           // axis-0 pass: 0 registers, 1 staged, 2 TMA, 3 TMA + registers
  // Float-pair arithmetic for bri17_apply_stiffness(_host) on FP64 handles
  // (df64.cuh); tables built on first enable.
  bool float_pair;
  int fused_form_df;
  void* table_df;
  bri17gb::Tables<bri17gb::df64> tabdf;
  // The mixed solvers' FP64 residuals (reliable updates) run in float pairs
  // (set by prepare_accurate_residual).
  bool residual_df;
  // Set around a CG iteration's operator application on an FP32 handle
  // (apply_stiffness_cg_async): the axis-0 pass sums p.Kp into this state.
  bri17gb::CgState* cg_st;
  double* cg_part;
  // Status words the handle's kernels set when a bounded device wait runs
  // out ([0]) or a tile is skipped ([1]): page-locked host memory mapped
  // into the device, read by the host without a copy.
  int* status_host;
  int* status_dev;
  // Per-mode calls on host buffers (bri17_modal_*_host, lazy): page-locked
  // staging mapped into the device, so a call is one kernel launch and one
  // synchronisation of a private stream; a lock, because those calls are
  // const in the C++ API and may come from several threads.
  unsigned char* mode_stage_host;
  unsigned char* mode_stage_dev;
  size_t mode_stage_bytes;
  cudaStream_t mode_stream;
  std::mutex* mode_mu;
};

namespace bri17gb {

constexpr int kHostEvents = 64;

// Scalar byte size of a handle's fields.
inline size_t scalar_bytes(const bri17_op* op) {
  return op->precision == BRI17_F64 ? sizeof(double) : sizeof(float);
}

// BRI17_OK when the current CUDA device is the handle's device.
int check_device(const bri17_op* op);

// BRI17_ERR_TIMEOUT, with the status words cleared, when one of the handle's
// kernels (or its FP32 twin's) recorded a bounded device wait that ran out,
// or a skipped tile, since the last call; else BRI17_OK.  Reads completed
// work only: call it after synchronising the streams the work ran on, or at
// entry to report an earlier call's failure.
int take_status(bri17_op* op);

// Grow the spectrum buffer to `comps` components.
int ensure_spectrum(bri17_op* op, int comps);

// Enqueue f = K u on `stream` for a handle of either precision.
int apply_stiffness_async(bri17_op* op, const void* u, void* f,
                          cudaStream_t stream);

// FP64-accurate f = K u for the mixed solvers' reliable updates.
// prepare_accurate_residual (called before a solve, outside any stream
// capture) builds the float-pair tables when the grid has float-pair
// instances, unless BRI17_MIXED_RESIDUAL=f64 (for measurements) or the
// handle is already in float pairs; apply_accurate_async then runs the
// float-pair operator (relative difference ~1e-14 from the FP64 operator, at
// about four times its speed on GB300), else the handle's own operator.
int prepare_accurate_residual(bri17_op* op);
int apply_accurate_async(bri17_op* op, const double* u, double* f, cudaStream_t stream);
// The same float-pair application with the material of one server slot:
// `mat_df` (device) holds (s, mu) as two float pairs (hi, lo each), the
// values the slot's FP64 residual would take from its (s, mu) doubles.
// Needs prepare_accurate_residual to have enabled float pairs.
int apply_accurate_mat_async(bri17_op* op, const double* u, double* f, const void* mat_df,
                             cudaStream_t stream);

// CG iterations on FP32 handles: whether the handle's stiffness pass can
// sum p.Kp by Parseval (3D power-of-two grid with an even last axis, the
// TMA-staged axis-0 form), and the application that does so into st->pq and
// st->alpha (one partial per axis-0 CTA in `part`, at least g.P entries).
bool cg_pq_fusable(const bri17_op* op);
int apply_stiffness_cg_async(bri17_op* op, const float* p, float* q, bri17gb::CgState* st,
                             double* part, cudaStream_t stream);

// Batched forms used by the server: `batch` fields of one geometry,
// contiguous (entry z at z * dim * size), with per-entry material
// (s, mu) pairs in `mat` (device, precision of the handle, already scaled by
// |h|/|N|).  spec must hold batch * dim * cspec complex values.  `flags`
// (optional, device) skips entry z when flags[z * flag_stride] == 0.
int apply_stiffness_batched_async(bri17_op* op, int batch, const void* u,
                                  void* f, void* spec, const void* mat,
                                  cudaStream_t stream, const int* flags = nullptr,
                                  int flag_stride = 0);
int eigenstress_rhs_batched_async(bri17_op* op, int batch, const void* tau,
                                  void* b, void* spec, cudaStream_t stream);

}  // namespace bri17gb
