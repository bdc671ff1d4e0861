// Launch interface between the host library and the kernels (fr_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include "fr_layout.h"

namespace fr {

// Hitpoint records of one iteration, one per pixel (SoA of float4):
//   pos   xyz position,          w type (int bits: kHitNone/kHitHit/kHitOnlyDirect)
//   nrm   xyz geometry normal,   w roughness
//   out   xyz outgoing dir,      w material id (int bits)
//   wgt   xyz pixel weight,      w facet id (int bits)
struct HitpointBuf {
  float4* pos;
  float4* nrm;
  float4* out;
  float4* wgt;
  float4* dl;            // this iteration's direct light per pixel (with an environment map)
  uint32_t* list;        // pixels holding a hitpoint this iteration, in no set order
  uint32_t* list_count;  // zeroed before the eye pass
};

// Photon slots: kPhotonSlots per path, persistent across iterations as the
// reference's photon deques are (SPPM.cpp:753).
//   pos  xyz position, w ray index of refraction
//   flux xyz flux,     w pdf
//   dir  xyz incoming direction, w 1 valid / 0 invalid
// Photon slots, slot-major: slot k of path i at k * paths + i, so that the
// emission's slot-0 stores and the grid's per-path reads are coalesced
// across a warp's consecutive paths.  A photon's id (the grid's dir.w, the
// path's importance) stays i * kPhotonSlots + k.
struct PhotonSlots {
  float4* pos;
  float4* flux;
  float4* dir;
  uint32_t paths;  // slot stride: the photon paths of the context (photons of a radius query)
};

// Photons sorted by cell of the hashed grid; dir.w holds the source slot id.
struct PhotonGrid {
  float4* pos;
  float4* flux;
  float4* dir;
  uint32_t* cell_count;  // [table]  photons per bucket (counted down to zero by the scatter)
  uint32_t* cell_start;  // [table + 1] exclusive prefix of cell_count
  uint32_t table;        // bucket count, power of two
};

// Wavefront passes (see fr_kernels.cu): per-path state, hit records, the two
// queues of live paths and the per-surface-type queues that the trace kernel
// sorts each round's hits into for the shade kernel.  qcount[r] counts the
// paths of round r; every counter is zeroed once per iteration.
// Rounds of trace/sort/shade before the tail kernel takes the paths still
// alive.  A round with few paths is bound by the latency of its slowest path
// and costs a launch sequence, while the tail advances each of its paths a
// bounce at the latency of one trace and shade; so a round r >= 1 with fewer
// than the pass's minimum of live paths is skipped (and with it every later
// round, which then has none) and the tail starts from it.  The maximum is
// reached only by scenes whose paths stay alive long (glass).
#ifndef FR_EYE_ROUNDS
#define FR_EYE_ROUNDS 8
#endif
#ifndef FR_PHOTON_ROUNDS
#define FR_PHOTON_ROUNDS 16
#endif
#ifndef FR_EYE_TAIL_MIN
#define FR_EYE_TAIL_MIN 0
#endif
#ifndef FR_PHOTON_TAIL_MIN
#define FR_PHOTON_TAIL_MIN 16384
#endif
constexpr int kEyeRounds = FR_EYE_ROUNDS;
constexpr int kPhotonRounds = FR_PHOTON_ROUNDS;
constexpr uint32_t kEyeTailMin = FR_EYE_TAIL_MIN;        // 0: every round runs
constexpr uint32_t kPhotonTailMin = FR_PHOTON_TAIL_MIN;
// In the captured iteration graph, photon rounds from this one on sit in
// conditional (IF) nodes, so skipped rounds launch nothing; the earlier ones
// are plain launches (skipping by themselves when they have too few paths).
constexpr int kPhotonGatedFrom = 5;
constexpr int kWaveRounds = kEyeRounds > kPhotonRounds ? kEyeRounds : kPhotonRounds;  // counter layout
constexpr int kShadeQueues = 5;  // one per surface type, then misses
struct PathWave {
  float4 *a, *b, *c, *d;  // path state
  float4* hit;            // u, v, triangle, facet (triangle -1: miss)
  uint32_t* queue[2];     // live paths of the current and the next round
  uint32_t* qcount;       // kWaveRounds + 2 counters
  uint32_t* mq;           // kShadeQueues queues of `cap` entries: this round's hits by surface type
  uint32_t* mcount;       // kWaveRounds * kShadeQueues counters
  uint32_t* tfetch;       // kWaveRounds counters: queue entries claimed by the trace kernel
  uint32_t cap;
  uint32_t min_live;      // rounds r >= 1 with fewer live paths go to the tail
};

// The round the tail kernel starts from, after at most `rounds` rounds (the
// host's copy of the rule the kernels apply to the counters).
inline int wave_tail_round(const uint32_t* qcount, int rounds, uint32_t min_live) {
  int r = rounds > 0 ? 1 : 0;
  while (r < rounds && qcount[r] >= min_live) ++r;
  return r;
}

// Per-pixel progressive state (SharedHitPoint, SPPM.h:112-126): tau in FP64.
struct PixelState {
  double* tau;    // [3 * pixels]
  int32_t* n;     // NumPhoton (int, truncating update, SPPM.cpp:447)
  float* r;       // Radius
  int32_t* g;     // NumGather
  float4* dl;     // DirectLight (xyz) and NumDirectLight (w, int bits)
};

// Scratch shared by the kernels of one iteration.
struct GridInfo {
  float cell;        // cell edge for this iteration
  float inv_cell;
  float origin[3];
  float r_sum;       // sum of radii of this iteration's hitpoints
  uint32_t r_count;  // number of this iteration's hitpoints
  uint32_t pad;
};

struct ScanTemp {
  uint32_t* level[4];     // block sums per level
  uint32_t level_n[4];
  int levels;
};

void upload_byte_lut(cudaStream_t s);

// Wavefront passes, launched round by round by the host: a start kernel,
// rounds of trace / sort / shade over the live-path queue, and a tail
// kernel.  `grid` is the block count of the persistent-style round kernels.
void launch_next_step(uint32_t* step, cudaStream_t s);
int pw_tail_blocks_per_sm();
void launch_ew_start(const CameraGPU& cam, const IterParams& it, PathWave w, cudaStream_t s);
// coherent: the queue holds rays in an order that neighbouring lanes should
// keep (camera rays in pixel order); otherwise lanes fetch rays dynamically.
void launch_wave_trace(const SceneGPU& sc, PathWave w, int round, int grid, bool coherent, int* err, cudaStream_t s);
void launch_wave_sort(const SceneGPU& sc, PathWave w, int round, int grid, cudaStream_t s);
void launch_round_gate(cudaGraphConditionalHandle h, const PathWave& w, int round, uint32_t* rounds_run,
                       cudaStream_t s);
void launch_ew_shade(const SceneGPU& sc, const IterParams& it, const float* rr_eye, PathWave w, HitpointBuf hp,
                     PixelState st, GridInfo* gi, int round, int grid, cudaStream_t s);
void launch_ew_tail(const SceneGPU& sc, const IterParams& it, const float* rr_eye, PathWave w, HitpointBuf hp,
                    PixelState st, GridInfo* gi, int round, int grid, int* err, cudaStream_t s);
void launch_pw_emit(const SceneGPU& sc, const IterParams& it, PhotonSlots ph, PathWave w, uint32_t* counts,
                    cudaStream_t s);
void launch_pw_shade(const SceneGPU& sc, const IterParams& it, PhotonSlots ph, PathWave w, uint32_t* counts,
                     int round, int grid, cudaStream_t s);
void launch_pw_tail(const SceneGPU& sc, const IterParams& it, PhotonSlots ph, PathWave w, uint32_t* counts,
                    int round, int grid, int* err, cudaStream_t s);
int photon_pass_blocks_per_sm();
// Points the kernels at the exact-value tables (see fr_bsdf.cuh).
void upload_tables(const float2* sincos_tab, const float* sqrt1m_tab, cudaStream_t s);
void launch_grid_setup(GridInfo* gi, const SceneGPU& sc, float cell_scale, float r0, cudaStream_t s);
// stride: slots per path (kPhotonSlots for the render loop, 1 for a flat photon list).
void launch_photon_count(PhotonSlots ph, const uint32_t* counts, int paths, int stride, PhotonGrid g,
                         const GridInfo* gi, cudaStream_t s);
// Returns the number of kernels launched.
int launch_scan(uint32_t* data_in, uint32_t* data_out, uint32_t n, ScanTemp& tmp, cudaStream_t s);
void launch_photon_scatter(PhotonSlots ph, const uint32_t* counts, int paths, int stride, PhotonGrid g,
                           const GridInfo* gi, cudaStream_t s);
// Words of block-sum scratch launch_scan needs for n elements; fills the level sizes of t.
uint32_t scan_temp_words(uint32_t n, ScanTemp& t);
// One warp per listed hitpoint; resident_blocks blocks of 256 threads.
// importance: per-path sums of the flux each path's photons bring to
// hitpoints (the guide's training signal, fixed point: importance_split in
// fr_guide.h), or nullptr.
void launch_gather_update(const SceneGPU& sc, const IterParams& it, HitpointBuf hp, PhotonGrid g, const GridInfo* gi,
                          PixelState st, int32_t* dbg_m, float4* dbg_phi, unsigned long long* importance,
                          int resident_blocks, cudaStream_t s);
int gather_blocks_per_sm();
// ExportPNG's resample and 8-bit quantization of a resolved image.
void launch_export_rgba8(const float4* img, int width, int height, uint32_t* out, cudaStream_t s);
// The N/tau/R update from given per-pixel photon counts and flux sums.
// float_n: N held as float bits (kFlagFloatPhotonCount).
void launch_update(PixelState st, const int32_t* m, const float4* phi, int pixels, float alpha, bool float_n,
                   cudaStream_t s);
void launch_resolve(PixelState st, int pixels, double photons_total, double iterations, bool standard, float4* out,
                    cudaStream_t s);

// Parity entry points.
void launch_trace_closest(const SceneGPU& sc, const float* rays, int n, int32_t* facet, float* tuv, int* err,
                          cudaStream_t s);
void launch_trace_any(const SceneGPU& sc, const float* rays, int n, int32_t* hit, int* err, cudaStream_t s);
// A ball that query_ball_ok refuses gets the count -1 and sets kErrQuery in
// *err when err is not NULL.
void launch_radius_count(const float4* hp_pos_r, int nh, PhotonGrid g, const GridInfo* gi, int32_t* m,
                         uint32_t* pairs, uint32_t pair_cap, uint32_t* pair_count, int* err, cudaStream_t s);

// Radius count with the fixed scratch of fr_noalloc.cu (allocates nothing).
int radius_count_noalloc(const float* hp_dev, int32_t nh, const float* photons_dev, int32_t np, float cell,
                         int32_t* counts_dev, cudaStream_t stream, const char** msg);

// Photon-emission guide (fr_guide.cu).
struct GuideGPU;
int guide_configure();  // opts the training kernel into its shared memory
void launch_pw_emit_guided(const SceneGPU& sc, const IterParams& it, PhotonSlots ph, PathWave w, uint32_t* counts,
                           const GuideGPU& g, cudaStream_t s);
int guide_train_smem();
int launch_guide_select_batch(const GuideGPU& g, int paths, cudaStream_t s);  // kernels launched
int launch_guide_steps(const GuideGPU& g, cudaStream_t s);                    // kernels launched
int launch_guide_publish(const GuideGPU& g, cudaStream_t s);                  // 0, or -1 on a copy error
void launch_guide_prepare(const GuideGPU& g, cudaStream_t s);
// Sample selection and the gradient sums only (no update).
void launch_guide_gradients(const GuideGPU& g, int paths, cudaStream_t s);
int guide_select_blocks(int paths);  // blocks of the sample selection (select_part words)
std::vector<float> guide_initial_params(uint32_t seed);

// Device check of the tcgen05 GEMM block (fr_tc_check.cu): max |error| of
// three products against a host GEMM.
int check_tc_gemm(uint32_t seed, double* max_err, const char** msg);

// Device check of the float paths of fr_exact.cuh (fr_exact_check.cu).
int check_exact_math(uint64_t samples, uint32_t seed, uint64_t* mismatches, uint64_t* fast_paths, const char** msg);

}  // namespace fr
