// engine_base.h -- precision-independent interface of one engine instance.
//
// A context owns up to two engines: an FP32 engine behind the
// reference-mirror calls (broad / narrow / prepare / avbd submit+read) and a
// world engine of the configured precision behind the fused step.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/dio_cuda.h"

namespace dio {

struct EngineBase {
    virtual ~EngineBase() = default;
    // reference-mirror calls
    virtual int broad_submit(const DioGpuBody* bodies, uint32_t n) = 0;
    virtual int pair_count(uint32_t* count) = 0;
    virtual int read_pairs(DioPair* out, uint32_t cap, uint32_t* n) = 0;
    virtual int narrow_submit_pairs(const DioGpuBody* bodies, uint32_t n, const DioPair* pairs, uint32_t np) = 0;
    virtual int narrow_submit(uint32_t np) = 0;
    virtual int narrow_read(DioContactOut* out, uint32_t cap, uint32_t* n) = 0;
    virtual int set_hull(const float* xyzw, uint32_t count) = 0;
    virtual int prepare_contacts(const DioGpuBody* bodies, const DioBodyState* state, uint32_t n,
                                 const DioContactOut* slots, uint32_t n_slots, const DioContact* prev, uint32_t n_prev,
                                 const DioContainer* container, const DioAvbdOptions* options, DioContact* out,
                                 uint32_t cap, uint32_t* m, uint32_t* offsets, uint32_t* indices,
                                 uint32_t index_cap) = 0;
    virtual int avbd_submit(const DioBodyState* state, const float* positions, const float* orientations, uint32_t n,
                            const DioContact* contacts, uint32_t m, const DioConstraint* constraints, uint32_t nj,
                            const uint32_t* offsets, const uint32_t* indices, const DioRunOptions* options) = 0;
    virtual int avbd_read(const DioAvbdResult* out) = 0;
    // fused world
    virtual int world_upload(const DioWorldDesc* desc) = 0;
    virtual int step(const DioAvbdOptions* options, uint32_t steps) = 0;
    virtual int step_async(const DioAvbdOptions* options, uint32_t steps) = 0;
    virtual int download_async(DioGpuBody* bodies, DioBodyState* state) = 0;
    virtual int sync_check() = 0;  // synchronise and report the device error flags
    virtual int set_state(const DioGpuBody* bodies, const DioBodyState* state) = 0;
    // set_state in two halves: _begin enqueues the copies, the unpacking and
    // the device check of the dynamic-body set; _end waits for that check and
    // rebuilds the dynamic-body list if the set changed
    virtual int set_state_begin(const DioGpuBody* bodies, const DioBodyState* state) = 0;
    virtual int set_state_end() = 0;
    // per-frame pose and velocity records (DioBodyMotion): upload, and the
    // enqueued read-back
    virtual int set_motion(const DioBodyMotion* motion) = 0;
    virtual int download_motion_async(DioBodyMotion* motion) = 0;
    virtual int download(DioGpuBody* bodies, DioBodyState* state) = 0;
    virtual int download_f64(double* positions, double* orientations) = 0;
    virtual int contacts(DioContact* out, uint32_t cap, uint32_t* m) = 0;
    virtual int colors(uint32_t* out, uint32_t cap, uint32_t* n) = 0;
    virtual int stats(DioStepStats* out) = 0;
    virtual int reset_timers() = 0;
    // device copy of the world's evolving state (poses, velocities, rows,
    // counters) and its restoration; used by the autotuner's trials
    virtual int snapshot() = 0;
    virtual int restore() = 0;
    virtual int export_transforms(uint32_t format, const float* scales, void* out, size_t stride) = 0;
    // host byte image of the whole world for checkpoint / resume
    virtual int checkpoint(void* out, size_t cap, size_t* size) = 0;
    virtual int resume(const void* in, size_t size) = 0;
    virtual int world_sizes(uint32_t* n, uint32_t* n_dyn, uint32_t* n_joints, uint32_t* n_scenes) = 0;
    virtual void set_stream(cudaStream_t s) = 0;
    virtual void set_config(const DioConfig& c) = 0;
    // every scene of the uploaded world fits the scene-chunk solve
    virtual bool chunk_solve_possible() const = 0;

    std::string err;
};

EngineBase* make_engine_f32(const DioCapacity& cap, cudaStream_t s, const DioConfig& cfg);
EngineBase* make_engine_split(const DioCapacity& cap, cudaStream_t s, const DioConfig& cfg);
EngineBase* make_engine_f64(const DioCapacity& cap, cudaStream_t s, const DioConfig& cfg);

}  // namespace dio
