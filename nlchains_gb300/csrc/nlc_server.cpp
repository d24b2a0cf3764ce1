// Request server: continuous batching of ensemble-integration requests on one GPU.
//
// Requests move queue -> admitted (by HBM budget) -> prepared -> running -> finished:
//   * a preparer thread builds each admitted request's plan (canonical launch shape; for dDNKG the
//     host eigensolve), allocates and uploads its state and takes the t = 0 diagnostics sample;
//   * the scheduler thread groups idle prepared requests by kernel class (model, parameters, dt,
//     launch shape) and launches each group on a free stream slot: one persistent batched launch of
//     the resident integrator advancing every member by its own kernel_batching steps (DNLS
//     requests run their own fused launch), then one diagnostics sample per member, then an event;
//   * completed events return their requests to idle (entropies appended, blow-ups flagged);
//     requests with all steps done are retired (final state and energies copied out, device memory
//     released), which lets queued requests in.
// There is no round barrier: fast groups keep cycling while slow ones run.  A request's chains see
// exactly the arithmetic of a launch of their own (the batched kernel only changes which block
// integrates which chain), so results are identical alone and in the mix.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>

#include "nlc_host.h"

using namespace nlc;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
	uint64_t id = 0;
	nlc_model model{};
	std::vector<double> masses;
	std::vector<uint8_t> mask;
	uint32_t batching = 1;
	uint64_t steps = 0;
	std::vector<double> host_in;    // initial state, then the final state
	size_t state_bytes = 0;
	size_t need_bytes = 0;          // device memory estimate used for admission

	nlc_plan *plan = nullptr;
	PlanInfo info;
	double2 *d_state = nullptr;
	double *d_diag = nullptr;       // [n] linenergies + [2] entropies
	double *h_diag = nullptr;       // pinned
	int stream_slot = 0;

	uint64_t t = 0;
	std::vector<double> entropies;  // {WT, INF} per sample
	std::vector<double> lin;
	int state = NLC_REQ_QUEUED;
	int error = NLC_OK;
	bool prepared = false;          // plan, state and t = 0 sample ready (set by the scheduler)
	bool in_flight = false;         // a launch group with this request is on the GPU
	double submit_ms = 0, start_ms = 0, finish_ms = 0;

	void release_device() {
		if (plan) nlc_plan_destroy(plan), plan = nullptr;
		cudaFree(d_state), d_state = nullptr;
		cudaFree(d_diag), d_diag = nullptr;
		cudaFreeHost(h_diag), h_diag = nullptr;
	}
};

// Class key of a batched launch: everything the kernel takes from its parameter bank.
struct ClassKey {
	int model, variant, lanes, sites, threads;
	uint64_t dt_bits, m_bits, alpha_bits, beta_bits;
	bool operator<(const ClassKey &o) const {
		return std::tie(model, variant, lanes, sites, threads, dt_bits, m_bits, alpha_bits, beta_bits) <
		       std::tie(o.model, o.variant, o.lanes, o.sites, o.threads, o.dt_bits, o.m_bits, o.alpha_bits,
		                o.beta_bits);
	}
};

uint64_t bits(double x) {
	uint64_t b;
	std::memcpy(&b, &x, 8);
	return b;
}

}  // namespace

struct nlc_server {
	nlc_server_config cfg{};
	Clock::time_point t0;
	std::mutex mu;
	std::condition_variable cv_work, cv_done;
	std::deque<std::unique_ptr<Request>> queue;      // submitted, waiting for budget
	std::deque<Request *> to_prepare;                  // admitted, plan being built
	std::vector<Request *> ready;                      // prepared, joins the next round
	std::map<uint64_t, std::unique_ptr<Request>> active;   // admitted (preparing or running)
	std::map<uint64_t, std::unique_ptr<Request>> finished;
	std::map<uint64_t, int> where;   // id -> NLC_REQ_* for lookups
	uint64_t next_id = 1;
	uint64_t used_bytes = 0;
	bool stop = false;
	std::thread worker, preparer;
	std::condition_variable cv_prepare;
	cudaStream_t prep_stream = nullptr;
	std::vector<cudaStream_t> streams;
	std::vector<cudaEvent_t> events;
	// per stream slot: the launch group on the GPU, its device job table and pinned staging
	std::vector<std::vector<Request *>> slot_reqs;
	std::vector<BatchJob *> d_tables;
	std::vector<size_t> d_table_cap;
	std::vector<BatchJob *> h_slot;
	std::vector<size_t> h_slot_cap;
	std::string fatal;

	double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
};

namespace {

int admit(nlc_server *S, Request &R) {
	int rc = cudaSetDevice(S->cfg.device) == cudaSuccess ? NLC_OK : set_error(NLC_ECUDA, "cudaSetDevice");
	if (rc) return rc;
	nlc_model m = R.model;
	m.masses = R.masses.empty() ? nullptr : R.masses.data();
	m.entropy_mask = R.mask.empty() ? nullptr : R.mask.data();
	m.flags |= NLC_FLAG_CANONICAL_SHAPE | NLC_FLAG_COMPACT_DIAG | NLC_FLAG_NO_TUNE;
	if ((rc = nlc_plan_create(&m, &R.plan))) return rc;
	plan_info(R.plan, &R.info);
	const size_t n = m.chain_length;
	if ((rc = cuda_status(cudaMalloc(&R.d_state, R.state_bytes), "cudaMalloc state"))) return rc;
	if ((rc = cuda_status(cudaMalloc(&R.d_diag, (n + 2) * sizeof(double)), "cudaMalloc"))) return rc;
	if ((rc = cuda_status(cudaMallocHost(&R.h_diag, (n + 2) * sizeof(double)), "cudaMallocHost"))) return rc;
	cudaStream_t st = S->prep_stream;
	if ((rc = cuda_status(cudaMemcpyAsync(R.d_state, R.host_in.data(), R.state_bytes, cudaMemcpyHostToDevice, st),
	                      "upload")))
		return rc;
	return NLC_OK;
}

int sample(nlc_server *S, Request &R, cudaStream_t st) {
	const size_t n = R.model.chain_length;
	int rc = nlc_linenergies(R.plan, R.d_state, R.d_diag, R.d_diag + n, st);
	if (rc) return rc;
	return cuda_status(cudaMemcpyAsync(R.h_diag, R.d_diag, (n + 2) * sizeof(double), cudaMemcpyDeviceToHost, st),
	                   "diagnostics copy");
}

void retire(nlc_server *S, std::unique_ptr<Request> R, int state, int error) {
	R->state = state;
	R->error = error;
	R->finish_ms = S->now_ms();
	R->release_device();
	if (R->need_bytes <= S->used_bytes) S->used_bytes -= R->need_bytes;
	S->where[R->id] = state;
	S->finished[R->id] = std::move(R);
}

BatchJob *class_table(nlc_server *S, size_t slot, size_t count) {
	if (S->d_tables.size() <= slot) S->d_tables.resize(slot + 1, nullptr), S->d_table_cap.resize(slot + 1, 0);
	if (S->d_table_cap[slot] < count) {
		cudaFree(S->d_tables[slot]);
		S->d_tables[slot] = nullptr;
		S->d_table_cap[slot] = 0;
		if (cudaMalloc(&S->d_tables[slot], std::max<size_t>(count, 16) * sizeof(BatchJob)) != cudaSuccess) return nullptr;
		S->d_table_cap[slot] = std::max<size_t>(count, 16);
	}
	return S->d_tables[slot];
}

// Builds plans (the dDNKG eigensystem can take a while on the host), allocates and uploads the
// state and takes the t = 0 sample, off the scheduler thread so that rounds keep running.
void preparer_loop(nlc_server *S) {
	cudaSetDevice(S->cfg.device);
	for (;;) {
		Request *R;
		{
			std::unique_lock<std::mutex> lk(S->mu);
			S->cv_prepare.wait(lk, [&] { return S->stop || !S->to_prepare.empty(); });
			if (S->stop) return;
			R = S->to_prepare.front();
			S->to_prepare.pop_front();
		}
		int rc = admit(S, *R);
		if (!rc) rc = sample(S, *R, S->prep_stream);
		if (!rc) rc = cuda_status(cudaStreamSynchronize(S->prep_stream), "request set-up");
		std::lock_guard<std::mutex> lk(S->mu);
		if (rc) {
			R->error = rc;
		} else {
			const size_t n = R->model.chain_length;
			R->entropies.push_back(R->h_diag[n]), R->entropies.push_back(R->h_diag[n + 1]);
			if (!std::isfinite(R->h_diag[n]) || !std::isfinite(R->h_diag[n + 1])) R->error = NLC_EBLOWUP;
		}
		S->ready.push_back(R);
		S->cv_work.notify_all();
	}
}

// Launch the next kernel_batching steps plus one sample for a group of idle requests of one class
// (several: one packed launch; one: its own plan's launch) on stream slot `slot`.
int launch_group(nlc_server *S, size_t slot, const std::vector<Request *> &reqs) {
	cudaStream_t st = S->streams[slot];
	int rc = NLC_OK;
	if (reqs.size() == 1 || reqs[0]->model.model == NLC_DNLS) {
		for (Request *R : reqs)
			if (!rc) rc = nlc_move(R->plan, R->d_state, R->batching, st);
	} else {
		if (S->h_slot_cap[slot] < reqs.size()) {
			cudaFreeHost(S->h_slot[slot]);
			S->h_slot[slot] = nullptr;
			S->h_slot_cap[slot] = 0;
			const size_t cap = std::max<size_t>(reqs.size(), 64);
			if ((rc = cuda_status(cudaMallocHost(&S->h_slot[slot], cap * sizeof(BatchJob)), "cudaMallocHost"))) return rc;
			S->h_slot_cap[slot] = cap;
		}
		BatchJob *h = S->h_slot[slot];
		unsigned long long units = 0;
		const int gpb = reqs[0]->info.shape.threads / reqs[0]->info.shape.lanes;
		for (size_t i = 0; i < reqs.size(); i++) {
			Request *R = reqs[i];
			h[i].state = R->d_state;
			h[i].mp2_site = R->info.args.mp2_site;
			h[i].unit_begin = units;
			h[i].n = R->model.chain_length;
			h[i].copies = R->model.copies;
			h[i].steps = R->batching;
			h[i].pad = 0;
			units += (R->model.copies + gpb - 1) / gpb;
		}
		BatchJob *d = class_table(S, slot, reqs.size());
		if (!d) return set_error(NLC_ENOMEM, "batch table");
		if ((rc = cuda_status(cudaMemcpyAsync(d, h, reqs.size() * sizeof(BatchJob), cudaMemcpyHostToDevice, st),
		                      "batch table copy")))
			return rc;
		RealArgs a = reqs[0]->info.args;
		a.batch = d, a.nbatch = int(reqs.size()), a.batch_units = units;
		RealShape sh = reqs[0]->info.shape;
		int per_sm = 0;
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(
		    &per_sm, real_move_kernel(reqs[0]->info.model, reqs[0]->info.variant, sh.sites), sh.threads, 0);
		sh.blocks = int(std::min<unsigned long long>(units, (unsigned long long) std::max(per_sm, 1) * reqs[0]->info.sms));
		if ((rc = cuda_status(launch_real_move_batch(reqs[0]->info.model, reqs[0]->info.variant, sh, a, st),
		                      "batched move launch")))
			return rc;
	}
	for (Request *R : reqs)
		if (!rc) rc = sample(S, *R, st);
	if (!rc) rc = cuda_status(cudaEventRecord(S->events[slot], st), "cudaEventRecord");
	return rc;
}

// Event-driven scheduler: admits requests, launches every group of idle same-class requests on a
// free stream slot, and retires groups whose event has completed.  No round barrier: a group of
// small fast requests goes round after round while a large one is still on the GPU.
void worker_loop(nlc_server *S) {
	cudaSetDevice(S->cfg.device);
	const size_t nslots = S->streams.size();
	for (;;) {
		bool progressed = false;
		{
			std::unique_lock<std::mutex> lk(S->mu);
			auto admissible = [&] {
				if (S->queue.empty() || S->active.size() >= size_t(S->cfg.max_active)) return false;
				return S->active.empty() || S->used_bytes + S->queue.front()->need_bytes <= S->cfg.hbm_budget_bytes;
			};
			auto in_flight = [&] {
				for (auto &g : S->slot_reqs)
					if (!g.empty()) return true;
				return false;
			};
			auto idle_work = [&] {
				for (auto &kv : S->active) {
					const Request &R = *kv.second;
					if (R.prepared && !R.in_flight) return true;
				}
				return false;
			};
			auto free_slot = [&] {
				for (auto &g : S->slot_reqs)
					if (g.empty()) return true;
				return false;
			};
			// idle requests only need the scheduler when a slot is free (or they are to be retired)
			auto wake = [&] { return S->stop || admissible() || !S->ready.empty() || (idle_work() && free_slot()); };
			if (in_flight()) S->cv_work.wait_for(lk, std::chrono::microseconds(100), wake);
			else S->cv_work.wait(lk, wake);
			if (S->stop) return;
			// admission by HBM budget (first come, first served; a request larger than the whole
			// budget is admitted alone when nothing else is admitted)
			bool admitted = false;
			while (admissible()) {
				std::unique_ptr<Request> P = std::move(S->queue.front());
				S->queue.pop_front();
				S->used_bytes += P->need_bytes;
				S->where[P->id] = NLC_REQ_RUNNING;
				P->state = NLC_REQ_RUNNING;
				P->start_ms = S->now_ms();
				S->to_prepare.push_back(P.get());
				S->active[P->id] = std::move(P);
				admitted = true;
			}
			if (admitted) S->cv_prepare.notify_all();
			for (Request *R : S->ready) R->prepared = true;
			S->ready.clear();
		}

		// 1. completed groups: record their samples
		std::vector<Request *> finished;
		for (size_t slot = 0; slot < nslots; slot++) {
			auto &g = S->slot_reqs[slot];
			if (g.empty()) continue;
			const cudaError_t e = cudaEventQuery(S->events[slot]);
			if (e == cudaErrorNotReady) continue;
			std::lock_guard<std::mutex> lk(S->mu);
			if (e != cudaSuccess) {
				S->fatal = cudaGetErrorString(e);
				for (Request *R : g) R->error = NLC_ECUDA;
			}
			for (Request *R : g) {
				R->in_flight = false;
				if (R->error) continue;
				const size_t n = R->model.chain_length;
				R->t += R->batching;
				R->entropies.push_back(R->h_diag[n]), R->entropies.push_back(R->h_diag[n + 1]);
				if (!std::isfinite(R->h_diag[n]) || !std::isfinite(R->h_diag[n + 1])) R->error = NLC_EBLOWUP;
			}
			g.clear();
			progressed = true;
		}

		// 2. retire finished / failed idle requests, and group the idle ones with steps left
		std::map<ClassKey, std::vector<Request *>> classes;
		std::vector<std::vector<Request *>> singles;
		{
			std::lock_guard<std::mutex> lk(S->mu);
			for (auto &kv : S->active) {
				Request *R = kv.second.get();
				if (!R->prepared || R->in_flight) continue;
				if (R->error || R->t >= R->steps) {
					finished.push_back(R);
					continue;
				}
				if (R->model.model == NLC_DNLS) {
					singles.push_back({R});
					continue;
				}
				const PlanInfo &I = R->info;
				ClassKey key{I.model, I.variant, I.shape.lanes, I.shape.sites, I.shape.threads, bits(R->model.dt),
				             bits(R->model.m), bits(R->model.alpha), bits(R->model.beta)};
				classes[key].push_back(R);
			}
		}
		for (Request *R : finished) {
			// final state and energies; copies outside the lock
			const size_t n = R->model.chain_length;
			if (R->d_state && R->error != NLC_ECUDA) {
				cudaMemcpy(R->host_in.data(), R->d_state, R->state_bytes, cudaMemcpyDeviceToHost);
				R->lin.assign(R->h_diag, R->h_diag + n);
			}
			std::lock_guard<std::mutex> lk(S->mu);
			auto it = S->active.find(R->id);
			std::unique_ptr<Request> P = std::move(it->second);
			S->active.erase(it);
			const int err = P->error;
			retire(S, std::move(P), err ? NLC_REQ_FAILED : NLC_REQ_DONE, err);
			progressed = true;
		}
		if (!finished.empty()) S->cv_done.notify_all();

		// 3. launch the groups on free slots (largest groups first)
		std::vector<std::vector<Request *>> groups;
		for (auto &kv : classes) groups.push_back(kv.second);
		for (auto &g : singles) groups.push_back(g);
		std::stable_sort(groups.begin(), groups.end(),
		                 [](const std::vector<Request *> &a, const std::vector<Request *> &b) { return a.size() > b.size(); });
		size_t next = 0;
		for (size_t slot = 0; slot < nslots && next < groups.size(); slot++) {
			if (!S->slot_reqs[slot].empty()) continue;
			auto &g = groups[next++];
			const int rc = launch_group(S, slot, g);
			std::lock_guard<std::mutex> lk(S->mu);
			for (Request *R : g) {
				R->in_flight = true;
				if (rc) R->error = rc;
			}
			S->slot_reqs[slot] = g;
			progressed = true;
		}
		if (!progressed) std::this_thread::yield();
	}
}

}  // namespace

extern "C" int nlc_server_create(const nlc_server_config *config, nlc_server **out) {
	if (!out) return set_error(NLC_EINVAL, "server pointer is NULL");
	std::unique_ptr<nlc_server> S(new nlc_server);
	if (config) S->cfg = *config;
	if (S->cfg.max_active <= 0) S->cfg.max_active = 256;
	if (S->cfg.streams <= 0) S->cfg.streams = 16;
	int rc = cuda_status(cudaSetDevice(S->cfg.device), "cudaSetDevice");
	if (rc) return rc;
	if (!S->cfg.hbm_budget_bytes) {
		size_t fr = 0, tot = 0;
		if ((rc = cuda_status(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo"))) return rc;
		S->cfg.hbm_budget_bytes = uint64_t(fr * 0.6);
	}
	for (int i = 0; i < S->cfg.streams; i++) {
		cudaStream_t st;
		cudaEvent_t ev;
		if ((rc = cuda_status(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
		S->streams.push_back(st);
		if ((rc = cuda_status(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate"))) return rc;
		S->events.push_back(ev);
	}
	if ((rc = cuda_status(cudaStreamCreateWithFlags(&S->prep_stream, cudaStreamNonBlocking), "cudaStreamCreate")))
		return rc;
	S->slot_reqs.resize(S->streams.size());
	S->d_tables.assign(S->streams.size(), nullptr);
	S->d_table_cap.assign(S->streams.size(), 0);
	S->h_slot.assign(S->streams.size(), nullptr);
	S->h_slot_cap.assign(S->streams.size(), 0);
	S->t0 = Clock::now();
	nlc_server *raw = S.get();
	S->worker = std::thread([raw] { worker_loop(raw); });
	S->preparer = std::thread([raw] { preparer_loop(raw); });
	*out = S.release();
	return NLC_OK;
}

extern "C" int nlc_server_destroy(nlc_server *S) {
	if (!S) return NLC_OK;
	{
		std::lock_guard<std::mutex> lk(S->mu);
		S->stop = true;
	}
	S->cv_work.notify_all();
	S->cv_prepare.notify_all();
	if (S->worker.joinable()) S->worker.join();
	if (S->preparer.joinable()) S->preparer.join();
	cudaSetDevice(S->cfg.device);
	if (S->prep_stream) cudaStreamSynchronize(S->prep_stream), cudaStreamDestroy(S->prep_stream);
	for (cudaStream_t st : S->streams) cudaStreamSynchronize(st);
	for (auto &kv : S->active) kv.second->release_device();
	for (BatchJob *p : S->d_tables) cudaFree(p);
	for (BatchJob *p : S->h_slot) cudaFreeHost(p);
	for (cudaStream_t st : S->streams) cudaStreamDestroy(st);
	for (cudaEvent_t ev : S->events) cudaEventDestroy(ev);
	delete S;
	return NLC_OK;
}

extern "C" int nlc_server_submit(nlc_server *S, const nlc_model *model, uint32_t batching, uint64_t steps,
                                 const void *host_state, uint64_t *id) {
	if (!S || !model || !host_state || !id) return set_error(NLC_EINVAL, "NULL argument");
	if (!batching) return set_error(NLC_EINVAL, "--kernel_batching must be a positive number");
	if (steps % batching) return set_error(NLC_EINVAL, "--steps must be a multiple of --kernel_batching");
	if (model->chain_length < 2 || !model->copies || !(model->dt > 0))
		return set_error(NLC_EINVAL, "--chain_length must be >= 2, --copies, --dt must be positive numbers");
	if (model->model == NLC_DDNKG && !model->masses) return set_error(NLC_EINVAL, "dDNKG needs the per-site masses");
	std::unique_ptr<Request> R(new Request);
	R->model = *model;
	const size_t n = model->chain_length;
	if (model->masses) R->masses.assign(model->masses, model->masses + n);
	if (model->entropy_mask) R->mask.assign(model->entropy_mask, model->entropy_mask + n);
	R->model.masses = nullptr, R->model.entropy_mask = nullptr;
	R->batching = batching;
	R->steps = steps;
	R->state_bytes = n * model->copies * sizeof(double2);
	const double *src = static_cast<const double *>(host_state);
	R->host_in.assign(src, src + 2 * n * model->copies);
	// state + diagnostics partial rows (<= one row block per SM) + tables
	R->need_bytes = R->state_bytes + size_t(4 * 160) * n * sizeof(double) + 16 * n * sizeof(double) +
	                (model->model == NLC_DDNKG ? n * n * sizeof(double) : 0) + (1 << 16);
	std::lock_guard<std::mutex> lk(S->mu);
	if (!S->fatal.empty()) return set_error(NLC_ECUDA, "server stopped after a CUDA error: " + S->fatal);
	R->id = S->next_id++;
	R->submit_ms = S->now_ms();
	*id = R->id;
	S->where[R->id] = NLC_REQ_QUEUED;
	S->queue.push_back(std::move(R));
	S->cv_work.notify_all();
	return NLC_OK;
}

static Request *lookup(nlc_server *S, uint64_t id) {
	for (auto &p : S->queue)
		if (p->id == id) return p.get();
	auto a = S->active.find(id);
	if (a != S->active.end()) return a->second.get();
	auto f = S->finished.find(id);
	if (f != S->finished.end()) return f->second.get();
	return nullptr;
}

extern "C" int nlc_server_poll(nlc_server *S, uint64_t id, nlc_request_status *st) {
	if (!S || !st) return set_error(NLC_EINVAL, "NULL argument");
	std::lock_guard<std::mutex> lk(S->mu);
	Request *R = lookup(S, id);
	if (!R) return set_error(NLC_ENOTFOUND, "no such request");
	st->state = R->state;
	st->error = R->error;
	st->steps_done = R->t;
	st->samples = R->entropies.size() / 2;
	st->submit_ms = R->submit_ms, st->start_ms = R->start_ms, st->finish_ms = R->finish_ms;
	return NLC_OK;
}

extern "C" int nlc_server_wait(nlc_server *S, uint64_t id, int32_t timeout_ms) {
	if (!S) return set_error(NLC_EINVAL, "NULL argument");
	std::unique_lock<std::mutex> lk(S->mu);
	auto ready = [&] {
		auto it = S->where.find(id);
		return it == S->where.end() || it->second == NLC_REQ_DONE || it->second == NLC_REQ_FAILED || !S->fatal.empty();
	};
	if (timeout_ms < 0) S->cv_done.wait(lk, ready);
	else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
		return set_error(NLC_ETIMEDOUT, "request still running");
	if (S->where.find(id) == S->where.end()) return set_error(NLC_ENOTFOUND, "no such request");
	if (!S->fatal.empty()) return set_error(NLC_ECUDA, "server stopped after a CUDA error: " + S->fatal);
	return NLC_OK;
}

extern "C" int nlc_server_result(nlc_server *S, uint64_t id, void *host_state, double *lin, double *entropies,
                                 uint64_t *samples) {
	if (!S) return set_error(NLC_EINVAL, "NULL argument");
	std::lock_guard<std::mutex> lk(S->mu);
	auto it = S->finished.find(id);
	if (it == S->finished.end()) return set_error(NLC_ENOTFOUND, "request not finished (or unknown)");
	Request &R = *it->second;
	if (host_state) std::memcpy(host_state, R.host_in.data(), R.state_bytes);
	if (lin && !R.lin.empty()) std::memcpy(lin, R.lin.data(), R.lin.size() * sizeof(double));
	if (entropies) std::memcpy(entropies, R.entropies.data(), R.entropies.size() * sizeof(double));
	if (samples) *samples = R.entropies.size() / 2;
	const int err = R.error;
	S->finished.erase(it);
	S->where.erase(id);
	return err ? set_error(err, err == NLC_EBLOWUP ? "non-finite entropy" : "request failed") : NLC_OK;
}
