// server.h -- the serving form: a request loop with continuous batching.
//
// Requests (one solve of a resident mesh with new coefficients, b and x0)
// queue on the host; a server thread admits them into a running batch --
// one per solver family (PCG for symmetric, PBiCG for asymmetric systems) --
// between launches of the batch's captured K-iteration graph, while memory
// (an HBM budget on the in-flight working sets) and batch slots allow.  A
// member leaves the batch when it has converged; its solution is copied out
// and the request completes.  Per-system reductions do not depend on the
// batch, so a request's result is bit-identical alone and in any mix.
#pragma once
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

namespace mrg {

struct ServerStats {
    uint64_t submitted = 0, completed = 0;
    int running = 0, queued = 0;
    size_t inflight_bytes = 0, peak_inflight_bytes = 0;
    int peak_running = 0;
};

class Server {
public:
    // sym / asym: controls of the two families (asym may be null: no
    // asymmetric requests).  budget: bytes of in-flight working sets (0: no
    // limit beyond the context's).  max_active: members per running batch.
    Server(Ctx* ctx, const Controls& sym, const Controls* asym, size_t budget, int max_active);
    ~Server();

    // Queue a solve.  Host arrays must stay valid and unchanged until the
    // request completes (x_out receives the solution).
    uint64_t submit(Mesh* m, int asym, const double* diag, const double* upper, const double* lower,
                    const double* ibou, const double* iint, const double* b, const double* x0, double* x_out);
    // done: the request finished (its record is then released); returns
    // its status.  wait blocks up to timeout_ms (< 0: no limit).
    int poll(uint64_t id, bool* done, Perf* perf, double* latency_ms, std::string* err);
    int wait(uint64_t id, double timeout_ms, bool* done, Perf* perf, double* latency_ms, std::string* err);
    ServerStats stats();

private:
    struct Request {
        uint64_t id = 0;
        Mesh* mesh = nullptr;
        int fam = 0;
        const double *diag = nullptr, *upper = nullptr, *lower = nullptr, *ibou = nullptr, *iint = nullptr;
        const double *b = nullptr, *x0 = nullptr;
        double* x_out = nullptr;
        double t_submit = 0, t_done = 0;
        size_t charged = 0;
        int state = 0;   // 0 queued, 1 running, 2 done
        int status = 0;
        Perf perf;
        std::string err;
    };
    struct Slot {
        double* d_bx = nullptr;   // caller-numbered b and x on the device
        size_t bytes = 0;         // measured working set (0: not yet measured)
        bool busy = false;        // a step of this mesh is in flight
    };
    struct Family {
        Controls cfg;
        bool enabled = false;
        BatchHost main, sub, fb, adm;
        std::vector<Request*> running;   // in main (the family's precision)
        std::vector<Request*> fbrun;     // in fb: mixed solves finishing in FP64
        std::vector<Request*> joining;   // prepared on the side stream, join main next
    };

    Ctx* ctx_;
    size_t budget_;
    int max_active_;
    Family fam_[2];
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<Request*> queue_;
    std::map<uint64_t, Request*> reqs_;
    std::map<Mesh*, Slot> slots_;
    uint64_t next_id_ = 1;
    bool stopping_ = false;
    ServerStats st_;
    cudaStream_t side_ = nullptr;      // admissions: uploads, views, factor, initial residual
    cudaEvent_t side_done_ = nullptr;
    std::thread thread_;
    // MRG_SERVER_PROFILE=1: host time by phase of the loop, printed to
    // stderr when the server is destroyed (idle: from the first drained
    // status of a pass to the next iteration launch)
    struct Prof {
        bool on = false;
        int passes = 0, rebuilds = 0;
        double idle = 0, iterate = 0, start = 0, harvest = 0, rebuild = 0, t_sync = 0;
    } prof_;

    void loop();
    void start(int f, std::vector<Request*>& reqs);
    bool harvest(int f);
    void finish(int f, std::vector<Request*>& done);
    void rebuild(int f);
    void fail_family(int f, int code, const std::string& msg);
    void complete(Request* r, int status, const std::string& err);
    size_t estimate(const Mesh& m) const;
};

}  // namespace mrg
