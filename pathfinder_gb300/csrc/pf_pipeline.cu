// Frames in flight: PFCUDAPipeline* (include/pathfinder_cuda.h).
//
// The CUDA level's counterpart of SceneProxy
// (renderer/src/concurrent/scene_proxy.rs:11-20, :86-121), which builds
// scenes on a worker thread and keeps a bounded number of render commands in
// flight.  Every stage of a frame here is GPU work, so what is kept in flight
// is whole frames: `depth` renderers, each owned by one worker thread, take
// the submitted frames from one queue in submission order.  A worker makes
// the same two calls a caller would (PFCUDASceneUpload, PFCUDARenderScene) on
// its own renderer, so each frame runs on its renderer's stream and the
// frames of different workers overlap on the GPU.  Host code only.
#include "pathfinder_cuda.h"

#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

struct PFCUDAPipeline {
    struct Job {
        uint64_t ticket;
        PFCUDASceneDesc scene;
        PFCUDABuildOptions options;
        bool has_options;
        int32_t width, height, out_memory;
        uint8_t* out;
    };
    std::vector<PFCUDARendererRef> renderers;
    std::vector<std::thread> workers;
    std::mutex m;
    std::condition_variable job_ready, job_done;
    std::deque<Job> queue;
    // submitted and not yet waited for: kPending until the frame is done;
    // `claimed` once a PFCUDAPipelineWait takes the ticket.  References to
    // the entries stay valid while the map grows.
    static constexpr int32_t kPending = -1;
    struct Entry {
        int32_t rc;
        bool claimed;
    };
    std::unordered_map<uint64_t, Entry> status;
    uint64_t next_ticket = 1;
    bool stopping = false;

    void work(PFCUDARendererRef r) {
        for (;;) {
            Job job;
            {
                std::unique_lock<std::mutex> lk(m);
                job_ready.wait(lk, [&] { return stopping || !queue.empty(); });
                if (queue.empty()) return;  // stopping, and every submitted frame taken
                job = queue.front();
                queue.pop_front();
            }
            int32_t rc = PFCUDASceneUpload(r, &job.scene);
            if (rc == PF_CUDA_OK)
                rc = PFCUDARenderScene(r, job.has_options ? &job.options : nullptr, job.width, job.height, job.out,
                                       job.out_memory);
            {
                std::lock_guard<std::mutex> lk(m);
                status.find(job.ticket)->second.rc = rc;  // entered at submission
            }
            job_done.notify_all();
        }
    }

    void stop() {
        {
            std::lock_guard<std::mutex> lk(m);
            stopping = true;
        }
        job_ready.notify_all();
        for (std::thread& t : workers)
            if (t.joinable()) t.join();
        workers.clear();
        for (PFCUDARendererRef r : renderers) PFCUDARendererDestroy(r);
        renderers.clear();
    }
};

extern "C" {

int32_t PFCUDAPipelineCreate(int32_t device, int32_t depth, const PFCUDARendererOptions* options,
                             PFCUDAPipelineRef* out) {
    if (!out || depth < 1 || depth > 64) return PF_CUDA_ERR_INVALID;
    *out = nullptr;
    // host allocation failures report PF_CUDA_ERR_LAUNCH, as the renderer's do
    PFCUDAPipeline* p = new (std::nothrow) PFCUDAPipeline();
    if (!p) return PF_CUDA_ERR_LAUNCH;
    for (int32_t i = 0; i < depth; i++) {
        PFCUDARendererRef r = nullptr;
        const int32_t rc = PFCUDARendererCreate(device, options, &r);
        if (rc != PF_CUDA_OK) {
            p->stop();
            delete p;
            return rc;
        }
        p->renderers.push_back(r);
    }
    try {
        for (PFCUDARendererRef r : p->renderers) p->workers.emplace_back([p, r] { p->work(r); });
    } catch (...) {
        p->stop();
        delete p;
        return PF_CUDA_ERR_LAUNCH;
    }
    *out = p;
    return PF_CUDA_OK;
}

int32_t PFCUDAPipelineDestroy(PFCUDAPipelineRef p) {
    if (!p) return PF_CUDA_ERR_INVALID;
    p->stop();
    delete p;
    return PF_CUDA_OK;
}

int32_t PFCUDAPipelineSubmit(PFCUDAPipelineRef p, const PFCUDASceneDesc* scene, const PFCUDABuildOptions* options,
                             int32_t width, int32_t height, uint8_t* out, int32_t out_memory, uint64_t* ticket) {
    if (!p || !scene || !out || !ticket || width <= 0 || height <= 0) return PF_CUDA_ERR_INVALID;
    PFCUDAPipeline::Job job{};
    job.scene = *scene;
    job.has_options = options != nullptr;
    if (options) job.options = *options;
    job.width = width;
    job.height = height;
    job.out = out;
    job.out_memory = out_memory;
    try {
        std::lock_guard<std::mutex> lk(p->m);
        if (p->stopping) return PF_CUDA_ERR_INVALID;
        job.ticket = p->next_ticket;
        p->status.emplace(job.ticket, PFCUDAPipeline::Entry{PFCUDAPipeline::kPending, false});
        try {
            p->queue.push_back(job);
        } catch (...) {
            p->status.erase(job.ticket);
            throw;
        }
        p->next_ticket++;
    } catch (...) {
        return PF_CUDA_ERR_LAUNCH;
    }
    p->job_ready.notify_one();
    *ticket = job.ticket;
    return PF_CUDA_OK;
}

int32_t PFCUDAPipelinePoll(PFCUDAPipelineRef p, uint64_t ticket, int32_t* done) {
    if (!p || !done) return PF_CUDA_ERR_INVALID;
    std::lock_guard<std::mutex> lk(p->m);
    const auto it = p->status.find(ticket);
    if (it == p->status.end() || it->second.claimed) return PF_CUDA_ERR_INVALID;
    *done = it->second.rc != PFCUDAPipeline::kPending ? 1 : 0;
    return PF_CUDA_OK;
}

int32_t PFCUDAPipelineWait(PFCUDAPipelineRef p, uint64_t ticket) {
    if (!p) return PF_CUDA_ERR_INVALID;
    std::unique_lock<std::mutex> lk(p->m);
    const auto it = p->status.find(ticket);
    if (it == p->status.end() || it->second.claimed) return PF_CUDA_ERR_INVALID;
    PFCUDAPipeline::Entry& e = it->second;  // only the claiming call erases it
    e.claimed = true;
    p->job_done.wait(lk, [&] { return e.rc != PFCUDAPipeline::kPending; });
    const int32_t rc = e.rc;
    p->status.erase(ticket);
    return rc;
}

}  // extern "C"
