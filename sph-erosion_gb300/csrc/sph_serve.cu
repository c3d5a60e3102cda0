// Request server: continuous batching of erosion scenes on one GPU.
//
// Requests are admitted against an HBM budget (and an optional cap on
// resident particles) at the boundary of each chunk of batched steps.  Each
// admitted request becomes a scene of one System with its own step budget,
// so scenes that arrive while others are on the GPU join the next chunk's
// launches, run alongside the others and retire independently.  A scene's
// results never depend on what it shares the GPU with: each scene's work is
// a separate set of tiles with its own neighbour ranges.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sph_erosion.h"
#include "sph_engine.h"
#include "sph_recipe.h"

namespace sph {

using Clock = std::chrono::steady_clock;

// Host-side inputs of a request's scene: parameters, particles, terrain.
struct PreparedScene {
    sph_params p;
    int particles = 0, side = 0;
    std::vector<float> pos, hgt;
};

static PreparedScene prepare_scene(const sph_params& base, const sph_request& r, int fbm_threads) {
    PreparedScene ps;
    RecipeGeometry g;
    recipe_geometry(r, base.smoothing_radius, &g);
    recipe_params(base, g, &ps.p);
    ps.particles = r.particles;
    ps.side = r.terrain_side;
    ps.pos.resize((size_t)r.particles * 3);
    recipe_particles(r, g, ps.pos.data());
    ps.hgt.resize((size_t)r.terrain_side * r.terrain_side);
    fbm_heights(r.seed, r.terrain_side, r.terrain_side, 6, g.amplitude, 2.0f, 0.5f, 0, ps.hgt.data(), fbm_threads);
    return ps;
}

static int create_prepared(System& sys, const PreparedScene& ps) {
    const int id = sys.create_scene(ps.p, ps.particles, ps.side, ps.side);
    try {
        sys.set_terrain(id, ps.side, ps.side, ps.hgt.data());
        sys.set_particles(id, ps.particles, ps.pos.data(), nullptr);
    } catch (...) {
        sys.destroy_scene(id);
        throw;
    }
    return id;
}

// Builds the scene of a request in `sys`; returns its id.
int scene_from_request(System& sys, const sph_params& base, const sph_request& r) {
    return create_prepared(sys, prepare_scene(base, r, 0));
}

class Server {
   public:
    explicit Server(const sph_server_config& c) : cfg_(c), sys_(sys_config(c)), t0_(Clock::now()) {
        if (cfg_.chunk_steps <= 0) cfg_.chunk_steps = 16;
        if (cfg_.hbm_budget <= 0) cfg_.hbm_budget = (int64_t)120 << 30;
        if (cfg_.cell_mult <= 0.0f) cfg_.cell_mult = 0.5f;
        if (cfg_.policy != 0 && cfg_.policy != 1) throw Error(SPH_ERR_INVALID, "policy must be 0 (arrival) or 1 (work)");
        cfg_.base.cell_mult = cfg_.cell_mult;
    }

    double now() const { return std::chrono::duration<double>(Clock::now() - t0_).count(); }
    void restart_clock() { t0_ = Clock::now(); }

    int64_t submit(const sph_request& r, double arrival) {
        if (r.particles <= 0 || r.steps < 0) throw Error(SPH_ERR_INVALID, "request needs particles > 0 and steps >= 0");
        // a request whose scene cannot fit even alone (without the optional
        // neighbour lists) is refused here, not left to block the queue
        if (request_bytes(r, false) > cfg_.hbm_budget)
            throw Error(SPH_ERR_CAPACITY, "the request's scene exceeds the whole HBM budget");
        Pending q{next_ticket_++, r, arrival, nullptr, 0};
        queue_.push_back(q);
        return q.ticket;
    }

    // One admission + chunk + retirement round.  Returns the number of
    // requests still queued or resident.
    // The chunk's steps run on the GPU while the host prepares the inputs of
    // requests that have arrived and are not yet admitted, so that the next
    // admission only uploads.
    int poll() {
        auto t = Clock::now();
        auto lap = [&](double* acc) {
            const auto u = Clock::now();
            *acc += std::chrono::duration<double>(u - t).count();
            t = u;
        };
        admit();
        lap(&stats_.admit_s);
        if (!active_.empty()) {
            sys_.step(cfg_.chunk_steps);
            prepare_ahead();
            lap(&stats_.prepare_s);
            sys_.sync();
            lap(&stats_.gpu_wait_s);
            ++chunks_;
            retire();
            lap(&stats_.retire_s);
        }
        return (int)(queue_.size() + ready_.size() + active_.size());
    }

    bool idle_until_arrival(double* next) const {
        if (!active_.empty() || !ready_.empty() || queue_.empty()) return false;
        *next = queue_.front().arrival;
        return true;
    }

    std::vector<sph_result>& done() { return done_; }
    const sph_server_stats& stats() const { return stats_; }
    sph_server_stats& stats() { return stats_; }

   private:
    struct Pending {
        int64_t ticket;
        sph_request req;
        double arrival;
        std::shared_ptr<PreparedScene> prep;  // filled ahead of admission
        int64_t held = 0;                     // host bytes of prep counted in prepared_bytes_
    };
    struct Active {
        Pending p;
        int scene;
        double admit;
        int64_t bytes;
    };

    static sph_system_config sys_config(const sph_server_config& c) {
        sph_system_config s;
        sph_system_config_default(&s);
        s.device = c.device;
        s.tile = c.tile > 0 ? c.tile : 256;
        s.graph_steps = c.chunk_steps > 0 ? c.chunk_steps : 16;
        s.hbm_budget = c.hbm_budget > 0 ? c.hbm_budget : ((int64_t)120 << 30);
        s.max_scenes = c.max_scenes > 0 ? c.max_scenes : 4096;
        if (c.variant > 0) s.variant = c.variant;
        // arenas start small and grow within the budget as requests arrive
        s.particle_capacity = 1 << 16;
        s.key_capacity = 1 << 18;
        s.terrain_capacity = 1 << 16;
        return s;
    }

    // Device bytes of a request's scene (validates the request's geometry).
    int64_t request_bytes(const sph_request& r, bool lists = true) {
        RecipeGeometry g;
        recipe_geometry(r, cfg_.base.smoothing_radius, &g);
        sph_params p;
        recipe_params(cfg_.base, g, &p);
        return sys_.scene_bytes(r.particles, r.terrain_side, r.terrain_side, p, lists);
    }

    void admit() {
        Range rg("sph/serve_admit");
        const double t = now();
        bool trimmed = false;
        collect_arrivals(t);
        while (!ready_.empty()) {
            const auto it = ready_.begin();
            Pending& q = it->second;
            const int64_t need = request_bytes(q.req);
            // with nothing resident a request is admitted even when its
            // lists do not fit (submit made sure the rest does): it then
            // runs without them
            if (reserved_ + need > cfg_.hbm_budget && !active_.empty()) break;
            if (cfg_.max_active_particles > 0 && !active_.empty() &&
                resident_particles_ + q.req.particles > cfg_.max_active_particles)
                break;
            int id;
            try {
                if (!q.prep) q.prep = std::make_shared<PreparedScene>(prepare_scene(cfg_.base, q.req, 0));
                id = create_prepared(sys_, *q.prep);
            } catch (const Error& e) {
                if (e.code == SPH_ERR_CAPACITY || e.code == SPH_ERR_NOMEM) {
                    if (!active_.empty()) break;  // wait for retirements to free arena space
                    if (!trimmed && sys_.trim()) {  // nothing resident: shrink the arenas, retry once
                        trimmed = true;
                        continue;
                    }
                    refuse(it, e.code);  // cannot fit even alone: retire it with its error
                    continue;
                }
                throw;
            }
            sys_.set_steps(id, q.req.steps);
            prepared_bytes_ -= q.held;
            active_.push_back(Active{Pending{q.ticket, q.req, q.arrival, nullptr, 0}, id, now(), need});
            reserved_ += need;
            resident_particles_ += q.req.particles;
            const bool retire_next = q.req.steps == 0;
            ready_.erase(it);
            stats_.peak_active = std::max<int32_t>(stats_.peak_active, (int32_t)active_.size());
            stats_.peak_particles = std::max<int64_t>(stats_.peak_particles, resident_particles_);
            stats_.peak_bytes = std::max<int64_t>(stats_.peak_bytes, sys_.memory_bytes());
            if (retire_next) break;  // retire it on the next round
        }
    }

    // Retire a request without running it: its result carries the error.
    void refuse(std::multimap<double, Pending>::iterator it, int code) {
        const Pending& q = it->second;
        sph_result r;
        std::memset(&r, 0, sizeof r);
        r.ticket = q.ticket;
        r.seed = q.req.seed;
        r.particles = q.req.particles;
        r.steps = q.req.steps;
        r.arrival_s = q.arrival;
        r.admit_s = r.done_s = now();
        r.status = code;
        prepared_bytes_ -= q.held;
        done_.push_back(r);
        ready_.erase(it);
    }

    // Move the requests that have arrived by time t into the ready set,
    // ordered by arrival (policy 0) or by work, particles x steps (policy 1).
    void collect_arrivals(double t) {
        while (!queue_.empty() && queue_.front().arrival <= t) {
            Pending& q = queue_.front();
            const double key = cfg_.policy == 1 ? (double)q.req.particles * (double)std::max(q.req.steps, 1)
                                                : q.arrival;
            ready_.emplace(key, std::move(q));
            queue_.pop_front();
        }
    }

    static int64_t prep_bytes(const Pending& q) {
        return q.prep ? (int64_t)(q.prep->pos.size() + q.prep->hgt.size()) * 4 : 0;
    }

    // Prepare, on host threads, the inputs of queued requests that have
    // arrived, in arrival order, up to kPrepareAhead requests or
    // kPrepareBytes of host memory held by prepared inputs.
    static constexpr int kPrepareAhead = 256;
    static constexpr int64_t kPrepareBytes = (int64_t)1 << 30;
    void prepare_ahead() {
        collect_arrivals(now());
        std::vector<Pending*> todo;
        int64_t bytes = prepared_bytes_;
        int held = 0;
        for (auto& kv : ready_) {
            Pending& q = kv.second;
            if (held >= kPrepareAhead || bytes >= kPrepareBytes) break;
            ++held;
            if (q.prep) continue;
            todo.push_back(&q);
            bytes += ((int64_t)q.req.particles * 3 + (int64_t)q.req.terrain_side * q.req.terrain_side) * 4;
        }
        if (todo.empty()) return;
        unsigned nt = std::thread::hardware_concurrency();
        nt = std::max(1u, std::min<unsigned>(nt ? nt : 1, (unsigned)todo.size()));
        std::vector<std::shared_ptr<PreparedScene>> out(todo.size());
        std::vector<std::thread> th;
        for (unsigned w = 0; w < nt; ++w)
            th.emplace_back([&, w] {
                for (size_t k = w; k < todo.size(); k += nt) {
                    try {
                        out[k] = std::make_shared<PreparedScene>(prepare_scene(cfg_.base, todo[k]->req, 1));
                    } catch (...) {
                        out[k] = nullptr;  // prepared again (and its error raised) at admission
                    }
                }
            });
        for (auto& x : th) x.join();
        for (size_t k = 0; k < todo.size(); ++k) {
            todo[k]->prep = out[k];
            todo[k]->held = prep_bytes(*todo[k]);
            prepared_bytes_ += todo[k]->held;
        }
    }

    // Retire every finished scene: one diagnostic launch for all of them
    // (mass units, FP64 energies and the state fingerprint), then free their
    // ranges for the next admission.
    void retire() {
        Range rg("sph/serve_retire");
        const double t = now();
        std::vector<Active> keep, fin;
        for (Active& a : active_) (sys_.steps(a.scene) > 0 ? keep : fin).push_back(a);
        if (!fin.empty()) {
            std::vector<int> ids(fin.size());
            for (size_t q = 0; q < fin.size(); ++q) ids[q] = fin[q].scene;
            std::vector<sph_diag> d(fin.size());
            sys_.diag_many(ids.data(), (int)ids.size(), d.data());
            for (size_t q = 0; q < fin.size(); ++q) {
                const Active& a = fin[q];
                sph_result r;
                std::memset(&r, 0, sizeof r);
                r.ticket = a.p.ticket;
                r.seed = a.p.req.seed;
                r.particles = a.p.req.particles;
                r.steps = a.p.req.steps;
                r.arrival_s = a.p.arrival;
                r.admit_s = a.admit;
                r.done_s = t;
                r.total_units = d[q].total_units;
                r.sediment_units = d[q].sediment_units;
                r.nan_particles = d[q].nan_particles;
                r.kinetic = d[q].kinetic;
                r.state_hash = d[q].state_hash;
                sys_.destroy_scene(a.scene);
                reserved_ -= a.bytes;
                resident_particles_ -= a.p.req.particles;
                done_.push_back(r);
                stats_.completed += 1;
                stats_.particle_steps += (double)a.p.req.particles * (double)a.p.req.steps;
            }
        }
        active_.swap(keep);
    }

    sph_server_config cfg_;
    System sys_;
    Clock::time_point t0_;
    std::deque<Pending> queue_;                // not yet arrived, by arrival time
    std::multimap<double, Pending> ready_;     // arrived, in admission order
    std::vector<Active> active_;
    std::vector<sph_result> done_;
    int64_t next_ticket_ = 1;
    int64_t reserved_ = 0;
    int64_t resident_particles_ = 0;
    int64_t prepared_bytes_ = 0;
    int chunks_ = 0;
    sph_server_stats stats_{};

   public:
    int chunks() const { return chunks_; }
};

}  // namespace sph

struct sph_server {
    sph::Server* srv;
};

namespace {

template <class F>
int serve_guard(F&& f) {
    try {
        f();
        return SPH_OK;
    } catch (const sph::Error& e) {
        sph::set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        sph::set_last_error("host allocation failed");
        return SPH_ERR_NOMEM;
    } catch (const std::exception& e) {
        sph::set_last_error(e.what());
        return SPH_ERR_INVALID;
    }
}

sph::Server& srv(sph_server* s) {
    if (!s || !s->srv) throw sph::Error(SPH_ERR_INVALID, "null server handle");
    return *s->srv;
}

}  // namespace

extern "C" {

SPH_API int sph_scene_from_request(sph_system* s, const sph_params* base, const sph_request* r, int* scene) {
    return serve_guard([&] {
        if (!s || !s->sys || !base || !r || !scene) throw sph::Error(SPH_ERR_INVALID, "null argument");
        *scene = sph::scene_from_request(*s->sys, *base, *r);
    });
}

SPH_API void sph_server_config_default(sph_server_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->tile = 256;
    c->cell_mult = 0.5f;
    c->chunk_steps = 16;
    c->hbm_budget = (int64_t)120 << 30;
    c->max_scenes = 4096;
    sph_params_default(&c->base);
}

SPH_API int sph_server_create(const sph_server_config* cfg, sph_server** out) {
    return serve_guard([&] {
        if (!out) throw sph::Error(SPH_ERR_INVALID, "null output handle");
        *out = nullptr;
        sph_server_config c;
        if (cfg)
            c = *cfg;
        else
            sph_server_config_default(&c);
        *out = new sph_server{new sph::Server(c)};
    });
}

SPH_API int sph_server_destroy(sph_server* s) {
    return serve_guard([&] {
        if (!s) return;
        delete s->srv;
        delete s;
    });
}

SPH_API int sph_server_submit(sph_server* s, const sph_request* r, int64_t* ticket) {
    return serve_guard([&] {
        if (!r) throw sph::Error(SPH_ERR_INVALID, "null request");
        sph::Server& S = srv(s);
        const int64_t t = S.submit(*r, S.now());
        if (ticket) *ticket = t;
    });
}

SPH_API int sph_server_poll(sph_server* s, sph_result* out, int cap, int* n_out, int* active) {
    return serve_guard([&] {
        sph::Server& S = srv(s);
        const int left = S.poll();
        auto& d = S.done();
        int k = 0;
        if (out && cap > 0) {
            k = std::min<int>(cap, (int)d.size());
            std::copy(d.begin(), d.begin() + k, out);
            d.erase(d.begin(), d.begin() + k);
        }
        if (n_out) *n_out = k;
        if (active) *active = left;
    });
}

SPH_API int sph_server_run_trace(sph_server* s, const sph_request* reqs, int n, sph_result* results,
                                 sph_server_stats* stats) {
    return serve_guard([&] {
        sph::Server& S = srv(s);
        if (n < 0 || (n > 0 && (!reqs || !results))) throw sph::Error(SPH_ERR_INVALID, "bad trace arguments");
        std::vector<int> order(n);
        for (int i = 0; i < n; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return reqs[a].arrival_s < reqs[b].arrival_s; });
        S.done().clear();
        S.stats() = sph_server_stats{};
        S.restart_clock();
        std::vector<int64_t> ticket_of(n);
        for (int k = 0; k < n; ++k) ticket_of[order[k]] = S.submit(reqs[order[k]], reqs[order[k]].arrival_s);
        const int chunks0 = S.chunks();
        for (;;) {
            const int left = S.poll();
            if (left == 0) break;
            double next;
            if (S.idle_until_arrival(&next)) {
                const double wait = next - S.now();
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
            }
        }
        std::vector<sph_result>& d = S.done();
        std::vector<double> lat;
        double first = 1e300, last = 0.0;
        for (const sph_result& r : d) {
            if (r.status != 0) continue;  // refused: not served
            lat.push_back(r.done_s - r.arrival_s);
            first = std::min(first, r.arrival_s);
            last = std::max(last, r.done_s);
        }
        for (int i = 0; i < n; ++i) {
            auto it = std::find_if(d.begin(), d.end(), [&](const sph_result& r) { return r.ticket == ticket_of[i]; });
            if (it == d.end()) throw sph::Error(SPH_ERR_STATE, "a request did not complete");
            results[i] = *it;
        }
        std::sort(lat.begin(), lat.end());
        sph_server_stats& st = S.stats();
        if (!lat.empty()) {
            auto rank = [&](double q) {
                size_t k = (size_t)std::ceil(q * (double)lat.size());
                return lat[std::min(lat.size() - 1, k > 0 ? k - 1 : 0)];
            };
            st.p50_s = rank(0.50);
            st.p99_s = rank(0.99);
            st.max_s = lat.back();
            st.wall_s = last - first;
            st.throughput = st.wall_s > 0 ? st.particle_steps / st.wall_s : 0.0;
        }
        st.chunks = S.chunks() - chunks0;
        if (stats) *stats = st;
        d.clear();
    });
}

}  // extern "C"
