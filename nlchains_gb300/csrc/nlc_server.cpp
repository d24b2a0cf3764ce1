// Request server: continuous batching of ensemble-integration requests on one GPU.
//
// Requests move queue -> admitted (by HBM budget) -> prepared -> running -> finished:
//   * four preparer threads build each admitted request's plan (smallest request first; canonical
//     launch shape, one block
//     per work unit; for dDNKG the host eigensolve) and allocate and upload its state, each on its own
//     high-priority stream; the t = 0 samples of newly prepared requests then go out as one group;
//   * the scheduler thread groups idle prepared requests by kernel class (model, parameters, dt,
//     launch shape) and launches each group, shortest remaining work first, on a free stream slot
//     of the group's priority band (four bands of stream priority: the GPU dispatches blocks of
//     nearly finished and short requests ahead of long ones): one batched launch of the
//     resident integrator advancing every member by its next segment (DNLS and windowed requests run
//     their own launches), then the diagnostics sample of every member whose round the segment
//     closes, then an event;
//   * a round of kernel_batching steps is cut into open segments so that no block lives much longer
//     than the quantum (3 ms): newly arrived work finds free SMs quickly (NLC_SEG_* flags: the
//     segments together run exactly the operations of one launch);
//   * completed events return their requests to idle (entropies appended, blow-ups flagged);
//     requests with all steps done are retired (final state and energies copied out, device memory
//     returned on a stream with no queued work), which lets queued requests in.
// There is no round barrier: fast groups keep cycling while slow ones run.  A request's chains see
// exactly the arithmetic of a launch of their own (the batched kernel only changes which block
// integrates which chain, segments only where a launch ends), so results are identical alone and
// in the mix.
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
	bool seeded = false;            // initial state generated on the device (nlc_initial_state)
	uint64_t seed = 0;
	double density = 0;
	std::vector<uint32_t> modes;
	size_t state_bytes = 0;
	size_t need_bytes = 0;          // device memory estimate used for admission
	double work = 0;                // site-steps of the request (weighted by model), orders set-up

	nlc_plan *plan = nullptr;
	PlanInfo info;
	double2 *d_state = nullptr;
	double *d_diag = nullptr;       // [n] linenergies + [2] entropies
	double *h_diag = nullptr;       // pinned
	int stream_slot = -1;           // slot of the request's last launch group (-1: the preparer's stream)

	uint64_t t = 0;                 // steps integrated
	uint32_t round_pos = 0;         // steps of the current round of `batching` steps already integrated
	uint32_t seg_steps = 0;         // steps of the launch in flight
	bool seg_samples = false;       // the launch in flight closes a round and takes its sample
	std::vector<double> entropies;  // {WT, INF} per sample
	std::vector<double> lin;
	int state = NLC_REQ_QUEUED;
	int error = NLC_OK;
	bool prepared = false;          // plan, state and t = 0 sample ready (set by the scheduler)
	bool in_flight = false;         // a launch group with this request is on the GPU
	bool sampled0 = false;          // the t = 0 diagnostics sample has been taken
	double submit_ms = 0, start_ms = 0, ready_ms = 0, finish_ms = 0;

	// device memory goes back in the order of `stream`: no device-wide wait.  The server passes a
	// stream with no queued work once the host has seen the request's last event complete, so the
	// memory is reusable at once; a free queued behind another group's kernel would hold up every
	// later allocation that reuses it.
	void release_device(cudaStream_t stream) {
		if (plan) plan_destroy_ordered(plan, stream), plan = nullptr;
		if (d_state) cudaFreeAsync(d_state, stream), d_state = nullptr;
		if (d_diag) cudaFreeAsync(d_diag, stream), d_diag = nullptr;
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
	std::thread worker;
	std::vector<std::thread> preparers;
	int prio_high = 0;
	std::condition_variable cv_prepare;
	cudaStream_t free_stream = nullptr;   // final read-backs and frees only: never holds queued kernels
	double quantum_us = 3000;
	std::vector<cudaStream_t> streams;
	std::vector<int> slot_band;   // priority band of each stream slot, 0 = the highest stream priority
	std::vector<cudaEvent_t> events;
	// per stream slot: the launch group on the GPU, its device job table and pinned staging
	std::vector<std::vector<Request *>> slot_reqs;
	std::vector<char> slot_sample_only;   // the group only takes the t = 0 samples
	std::vector<BatchJob *> d_tables;
	std::vector<size_t> d_table_cap;
	std::vector<BatchJob *> h_slot;
	std::vector<size_t> h_slot_cap;
	std::string fatal;
	// pinned read-back buffers, reused (cudaFreeHost would wait for the whole device)
	std::multimap<size_t, double *> pinned_free;
	std::vector<double *> pinned_all;

	double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
};

namespace {

double *pinned_get(nlc_server *S, size_t count) {
	size_t cap = 64;
	while (cap < count) cap <<= 1;
	{
		std::lock_guard<std::mutex> lk(S->mu);
		auto it = S->pinned_free.find(cap);
		if (it != S->pinned_free.end()) {
			double *p = it->second;
			S->pinned_free.erase(it);
			return p;
		}
	}
	double *p = nullptr;
	if (cudaMallocHost(&p, cap * sizeof(double)) != cudaSuccess) return nullptr;
	std::lock_guard<std::mutex> lk(S->mu);
	S->pinned_all.push_back(p);
	return p;
}

// caller holds S->mu
void pinned_put(nlc_server *S, double *p, size_t count) {
	if (!p) return;
	size_t cap = 64;
	while (cap < count) cap <<= 1;
	S->pinned_free.emplace(cap, p);
}

int admit(nlc_server *S, Request &R, cudaStream_t st) {
	int rc = cudaSetDevice(S->cfg.device) == cudaSuccess ? NLC_OK : set_error(NLC_ECUDA, "cudaSetDevice");
	if (rc) return rc;
	nlc_model m = R.model;
	m.masses = R.masses.empty() ? nullptr : R.masses.data();
	m.entropy_mask = R.mask.empty() ? nullptr : R.mask.data();
	m.flags |= NLC_FLAG_CANONICAL_SHAPE | NLC_FLAG_COMPACT_DIAG | NLC_FLAG_NO_TUNE | NLC_FLAG_SHARED_GPU;
	if ((rc = nlc_plan_create(&m, &R.plan))) return rc;
	plan_info(R.plan, &R.info);
	const size_t n = m.chain_length;
	if ((rc = cuda_status(cudaMallocAsync(&R.d_state, R.state_bytes, st), "cudaMallocAsync state"))) return rc;
	if ((rc = cuda_status(cudaMallocAsync(&R.d_diag, (n + 2) * sizeof(double), st), "cudaMallocAsync"))) return rc;
	if (!(R.h_diag = pinned_get(S, n + 2))) return set_error(NLC_ENOMEM, "pinned read-back buffer");
	if (R.seeded)
		return nlc_initial_state(R.plan, R.seed, 0, R.density, R.modes.data(), uint32_t(R.modes.size()), R.d_state, st);
	if ((rc = cuda_status(cudaMemcpyAsync(R.d_state, R.host_in.data(), R.state_bytes, cudaMemcpyHostToDevice, st),
	                      "upload")))
		return rc;
	return NLC_OK;
}

int sample(Request &R, cudaStream_t st) {
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
	R->release_device(S->free_stream);
	pinned_put(S, R->h_diag, R->model.chain_length + 2);
	R->h_diag = nullptr;
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
	// four preparers may each run an eigensolve: half the cores each (measured: large dDNKG requests
	// ready ~30% sooner than with a thread per core each, and no slower to serve)
	set_host_setup_threads(std::max(1u, host_setup_threads() / 2));
	// the dDNKG eigensystem on the host: on the GPU it would compete with the requests being served
	// (measured: 1.07x instead of 1.14x the alone path on the mixed stream)
	set_eigen_on_host(true);
	cudaSetDevice(S->cfg.device);
	cudaStream_t st = nullptr;
	if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, S->prio_high) != cudaSuccess) st = nullptr;
	for (;;) {
		Request *R;
		{
			std::unique_lock<std::mutex> lk(S->mu);
			S->cv_prepare.wait(lk, [&] { return S->stop || !S->to_prepare.empty(); });
			if (S->stop) {
				if (st) cudaStreamSynchronize(st), cudaStreamDestroy(st);
				return;
			}
			// the smallest admitted request first: a short request is not held behind the set-up of a
			// large one (a long host eigensolve, large tables)
			auto it = std::min_element(S->to_prepare.begin(), S->to_prepare.end(),
			                           [](const Request *a, const Request *b) { return a->work < b->work; });
			R = *it;
			S->to_prepare.erase(it);
		}
		int rc = st ? admit(S, *R, st) : set_error(NLC_ECUDA, "preparer stream");
		if (!rc) rc = cuda_status(cudaStreamSynchronize(st), "request set-up");
		std::lock_guard<std::mutex> lk(S->mu);
		if (rc) R->error = rc;
		R->ready_ms = S->now_ms();
		S->ready.push_back(R);
		S->cv_work.notify_all();
	}
}

// Estimated lifetime of one block per step in a launch of `blocks` blocks: k of them share an SM
// (at most the occupancy), and a block of fewer than four warps alone uses only part of the SM's
// four FP64 pipes.  ~3950 FP64 lane operations per SM and microsecond (600 G/s on 152 SMs).
double block_step_us(const PlanInfo &I, unsigned long long blocks) {
	const double k = std::min<double>(I.per_sm, std::max(1., std::ceil(double(blocks) / std::max(I.sms, 1))));
	const double pipes = std::min(4., k * I.block_warps) / 4;
	return I.block_ops * k / (3950. * pipes);
}

// Steps of the next launch of R: the rest of its round, or, when one block would then run longer
// than the quantum, an equal share of the rest that does not.
uint32_t segment_steps(const nlc_server *S, const Request &R, unsigned long long group_blocks) {
	const uint32_t left = R.batching - R.round_pos;
	const double est = block_step_us(R.info, group_blocks);
	if (S->quantum_us <= 0 || !(est > 0) || est * left <= S->quantum_us) return left;
	const uint32_t cap = uint32_t(std::max(1., std::floor(S->quantum_us / est)));
	const uint32_t parts = (left + cap - 1) / cap;
	return (left + parts - 1) / parts;
}

// Estimated GPU time of a request's remaining steps with the whole GPU to itself: FP64 work of a
// block's step times the blocks of one step, at ~3950 FP64 lane operations per SM and microsecond.
double remaining_us(const Request &R) {
	if (R.t >= R.steps) return 0.;
	const double blocks = std::max(R.info.grid, 1);
	return double(R.steps - R.t) * blocks * R.info.block_ops / (3950. * std::max(R.info.sms, 1));
}

// Priority band of a launch group from the least remaining work among its members: the GPU's block
// scheduler dispatches blocks of higher-priority streams first, so requests close to done (or short
// to begin with) are not held behind long ones -- shortest remaining work first, at block
// granularity.  Bands: < 20 ms, < 200 ms, < 2 s, longer.
int priority_band(const std::vector<Request *> &g) {
	double rem = 1e300;
	for (const Request *R : g) rem = std::min(rem, remaining_us(*R));
	return rem < 2e4 ? 0 : rem < 2e5 ? 1 : rem < 2e6 ? 2 : 3;
}

// Launch the next segment of every request of a group of idle requests of one class (several: one
// packed launch; one: its own plan's launch) on stream slot `slot`, plus the sample of each request
// whose round the segment closes.
int launch_group(nlc_server *S, size_t slot, const std::vector<Request *> &reqs) {
	NvtxRange r("server group");
	cudaStream_t st = S->streams[slot];
	int rc = NLC_OK;
	unsigned long long group_blocks = 0;
	for (Request *R : reqs) group_blocks += std::max(R->info.grid, 1);
	for (Request *R : reqs) {
		R->seg_steps = segment_steps(S, *R, group_blocks);
		R->seg_samples = R->round_pos + R->seg_steps == R->batching;
	}
	auto seg_flags = [](const Request &R) {
		return (R.round_pos ? NLC_SEG_CONTINUE : 0u) | (R.seg_samples ? 0u : NLC_SEG_OPEN);
	};
	if (reqs.size() == 1 || reqs[0]->model.model == NLC_DNLS || reqs[0]->info.windowed) {
		for (Request *R : reqs)
			if (!rc) rc = move_segment(R->plan, R->d_state, R->seg_steps, seg_flags(*R), st);
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
			h[i].steps = R->seg_steps;
			h[i].seg = seg_flags(*R);
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
		// one block per unit: blocks retire as they finish, so the groups on other streams interleave
		sh.blocks = int(std::min<unsigned long long>(units, 0x7fffffffull));
		if ((rc = cuda_status(launch_real_move_batch(reqs[0]->info.model, reqs[0]->info.variant, sh, a, st),
		                      "batched move launch")))
			return rc;
	}
	for (Request *R : reqs)
		if (!rc && R->seg_samples) rc = sample(*R, st);
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
			const bool sample_only = S->slot_sample_only[slot];
			for (Request *R : g) {
				R->in_flight = false;
				if (R->error) continue;
				const size_t n = R->model.chain_length;
				if (sample_only) {
					R->sampled0 = true;
				} else {
					R->t += R->seg_steps;
					R->round_pos += R->seg_steps;
					if (!R->seg_samples) continue;
					R->round_pos = 0;
				}
				R->entropies.push_back(R->h_diag[n]), R->entropies.push_back(R->h_diag[n + 1]);
				if (!std::isfinite(R->h_diag[n]) || !std::isfinite(R->h_diag[n + 1])) {
					const int st = plan_device_status(R->plan);   // a timed-out projection, else a blow-up
					R->error = st ? st : NLC_EBLOWUP;
				}
			}
			g.clear();
			progressed = true;
		}

		// 2. retire finished / failed idle requests, and group the idle ones with steps left
		std::map<ClassKey, std::vector<Request *>> classes;
		std::vector<std::vector<Request *>> singles;
		std::vector<Request *> first_samples;
		{
			std::lock_guard<std::mutex> lk(S->mu);
			for (auto &kv : S->active) {
				Request *R = kv.second.get();
				if (!R->prepared || R->in_flight) continue;
				if (!R->error && !R->sampled0) {
					first_samples.push_back(R);
					continue;
				}
				if (R->error || R->t >= R->steps) {
					finished.push_back(R);
					continue;
				}
				if (R->model.model == NLC_DNLS || R->info.windowed) {
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
				cudaMemcpyAsync(R->host_in.data(), R->d_state, R->state_bytes, cudaMemcpyDeviceToHost, S->free_stream);
				cudaStreamSynchronize(S->free_stream);
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
		// shortest remaining work first (ties: larger groups first)
		std::vector<std::pair<int, double>> urgency(groups.size());
		for (size_t i = 0; i < groups.size(); i++) {
			double rem = 1e300;
			for (const Request *R : groups[i]) rem = std::min(rem, remaining_us(*R));
			urgency[i] = {priority_band(groups[i]), rem};
		}
		std::vector<size_t> order(groups.size());
		for (size_t i = 0; i < order.size(); i++) order[i] = i;
		std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
			if (urgency[a].second != urgency[b].second) return urgency[a].second < urgency[b].second;
			return groups[a].size() > groups[b].size();
		});
		// a free slot of the wanted band, else of a lower priority, else any free slot
		auto pick_slot = [&](int band) {
			long best = -1;
			for (size_t slot = 0; slot < nslots; slot++) {
				if (!S->slot_reqs[slot].empty()) continue;
				const int b = S->slot_band[slot];
				if (b == band) return long(slot);
				if (best < 0 || (b > band && (S->slot_band[best] < band || b < S->slot_band[best]))) best = long(slot);
			}
			return best;
		};
		size_t next = 0;
		for (;;) {
			const bool sample_only = !first_samples.empty();
			if (!sample_only && next >= groups.size()) break;
			const long slot_l = pick_slot(sample_only ? 0 : urgency[order[next]].first);
			if (slot_l < 0) break;
			const size_t slot = size_t(slot_l);
			std::vector<Request *> g;
			int rc = NLC_OK;
			// the t = 0 samples of newly prepared requests go first, all in one group
			if (sample_only) {
				g.swap(first_samples);
				for (Request *R : g)
					if (!rc) rc = sample(*R, S->streams[slot]);
				if (!rc) rc = cuda_status(cudaEventRecord(S->events[slot], S->streams[slot]), "cudaEventRecord");
			} else {
				g = groups[order[next++]];
				rc = launch_group(S, slot, g);
			}
			S->slot_sample_only[slot] = sample_only;
			std::lock_guard<std::mutex> lk(S->mu);
			for (Request *R : g) {
				R->in_flight = true;
				R->stream_slot = int(slot);
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
	S->quantum_us = S->cfg.quantum_ms > 0 ? S->cfg.quantum_ms * 1e3 : S->cfg.quantum_ms < 0 ? 0. : 3000.;
	int rc = cuda_status(cudaSetDevice(S->cfg.device), "cudaSetDevice");
	if (rc) return rc;
	if (!S->cfg.hbm_budget_bytes) {
		size_t fr = 0, tot = 0;
		if ((rc = cuda_status(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo"))) return rc;
		S->cfg.hbm_budget_bytes = uint64_t(fr * 0.6);
	}
	// request set-up (plan, upload) runs on preparer streams of the highest priority: it gates latency
	int prio_low = 0, prio_high = 0;
	cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
	S->prio_high = prio_high;
	// launch slots in four priority bands (slot i in band i % 4), spread over the device's range
	for (int i = 0; i < S->cfg.streams; i++) {
		cudaStream_t st;
		cudaEvent_t ev;
		const int band = i % 4;
		const int prio = prio_high + int(std::lround(band * double(prio_low - prio_high) / 3.));
		if ((rc = cuda_status(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio), "cudaStreamCreate")))
			return rc;
		S->streams.push_back(st);
		S->slot_band.push_back(band);
		if ((rc = cuda_status(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate"))) return rc;
		S->events.push_back(ev);
	}
	if ((rc = cuda_status(cudaStreamCreateWithFlags(&S->free_stream, cudaStreamNonBlocking), "cudaStreamCreate")))
		return rc;
	// keep the memory returned by cudaFreeAsync cached in the device's pool between requests, and
	// never let an allocation silently wait for another stream's pending free (the pool grows instead)
	cudaMemPool_t pool;
	if (cudaDeviceGetDefaultMemPool(&pool, S->cfg.device) == cudaSuccess) {
		uint64_t threshold = UINT64_MAX;
		cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
		int internal = 0;
		cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &internal);
	}
	S->slot_reqs.resize(S->streams.size());
	S->slot_sample_only.assign(S->streams.size(), 0);
	S->d_tables.assign(S->streams.size(), nullptr);
	S->d_table_cap.assign(S->streams.size(), 0);
	S->h_slot.assign(S->streams.size(), nullptr);
	S->h_slot_cap.assign(S->streams.size(), 0);
	// job tables sized for max_active members up front: growing them later would synchronise
	for (size_t i = 0; i < S->streams.size(); i++) {
		const size_t cap = size_t(S->cfg.max_active);
		if ((rc = cuda_status(cudaMalloc(&S->d_tables[i], cap * sizeof(BatchJob)), "cudaMalloc"))) return rc;
		if ((rc = cuda_status(cudaMallocHost(&S->h_slot[i], cap * sizeof(BatchJob)), "cudaMallocHost"))) return rc;
		S->d_table_cap[i] = S->h_slot_cap[i] = cap;
	}
	S->t0 = Clock::now();
	nlc_server *raw = S.get();
	S->worker = std::thread([raw] { worker_loop(raw); });
	for (int i = 0; i < 4; i++) S->preparers.emplace_back([raw] { preparer_loop(raw); });
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
	for (auto &th : S->preparers)
		if (th.joinable()) th.join();
	cudaSetDevice(S->cfg.device);
	for (cudaStream_t st : S->streams) cudaStreamSynchronize(st);
	for (auto &kv : S->active) kv.second->release_device(S->free_stream);
	cudaDeviceSynchronize();
	if (S->free_stream) cudaStreamDestroy(S->free_stream);
	for (double *p : S->pinned_all) cudaFreeHost(p);
	for (BatchJob *p : S->d_tables) cudaFree(p);
	for (BatchJob *p : S->h_slot) cudaFreeHost(p);
	for (cudaStream_t st : S->streams) cudaStreamDestroy(st);
	for (cudaEvent_t ev : S->events) cudaEventDestroy(ev);
	delete S;
	return NLC_OK;
}

namespace {
// a request whose initial state is `host_state` (uploaded) or, with host_state NULL, the seeded
// ensemble of `seed_spec` (generated on the device by its preparer)
struct SeedSpec {
	uint64_t seed;
	double density;
	const uint32_t *modes;
	uint32_t nmodes;
};

int submit(nlc_server *S, const nlc_model *model, uint32_t batching, uint64_t steps, const void *host_state,
           const SeedSpec *seed_spec, uint64_t *id) {
	if (!S || !model || !id || (!host_state && !seed_spec)) return set_error(NLC_EINVAL, "NULL argument");
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
	// rough FP64 cost per site-step against DNKG's: Toda's exp 2.4x, DNLS's stencils ~10x (its
	// transforms ~15x)
	const double dnls = (model->flags & NLC_FLAG_DNLS_FOURIER) ? 15. : 10.;
	R->work = double(n) * model->copies * double(steps) *
	          (model->model == NLC_DNLS ? dnls : model->model == NLC_TODA ? 2.4 : 1.);
	if (host_state) {
		const double *src = static_cast<const double *>(host_state);
		R->host_in.assign(src, src + 2 * n * model->copies);
	} else {
		if (!seed_spec->nmodes || !seed_spec->modes || !(seed_spec->density > 0))
			return set_error(NLC_EINVAL, "a seeded request needs modes and a positive density");
		for (uint32_t j = 0; j < seed_spec->nmodes; j++)
			if (seed_spec->modes[j] >= n) return set_error(NLC_EINVAL, "mode index >= chain_length");
		R->seeded = true;
		R->seed = seed_spec->seed, R->density = seed_spec->density;
		R->modes.assign(seed_spec->modes, seed_spec->modes + seed_spec->nmodes);
		R->host_in.resize(2 * n * model->copies);   // receives the final state
	}
	// state + diagnostics partial rows (<= one row block per SM) + tables
	R->need_bytes = R->state_bytes + size_t(4 * 160) * n * sizeof(double) + 16 * n * sizeof(double) +
	                (model->model == NLC_DDNKG ? n * n * sizeof(double) : 0) + (1 << 16) +
	                (n > 4096 ? R->state_bytes : 0);   // windowed integrators: a second state buffer
	if (n > 4096) R->need_bytes += R->state_bytes + size_t(2 * 1024) * 4 * n * sizeof(double2);   // windows / FFT scratch
	if (model->model == NLC_DDNKG) {
		// the tensor-core projection (the plan's rule): BF16 slices of the state and of the
		// eigenvectors, and with 7 slices the first sweep's integer sums
		const bool bf16x3 = model->flags & NLC_FLAG_BF16X3_PROJECTION;
		if (bf16x3 || (model->flags & NLC_FLAG_TENSOR_PROJECTION) || (n >= 128 && !(model->flags & NLC_FLAG_FP64_PROJECTION))) {
			const size_t mp = (2ull * model->copies + 127) / 128 * 128, np = (size_t(n) + 127) / 128 * 128,
			             kp = (size_t(n) + 15) / 16 * 16, slices = bf16x3 ? 3 : 7;
			R->need_bytes += slices * (mp + np) * kp * 2 + (bf16x3 ? 0 : mp * np * 8);
		}
	}
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

}  // namespace

extern "C" int nlc_server_submit(nlc_server *S, const nlc_model *model, uint32_t batching, uint64_t steps,
                                 const void *host_state, uint64_t *id) {
	if (!host_state) return set_error(NLC_EINVAL, "NULL argument");
	return submit(S, model, batching, steps, host_state, nullptr, id);
}

extern "C" int nlc_server_submit_seeded(nlc_server *S, const nlc_model *model, uint32_t batching, uint64_t steps,
                                        uint64_t seed, double density, const uint32_t *modes, uint32_t nmodes,
                                        uint64_t *id) {
	const SeedSpec spec{seed, density, modes, nmodes};
	return submit(S, model, batching, steps, nullptr, &spec, id);
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
	st->submit_ms = R->submit_ms, st->start_ms = R->start_ms, st->ready_ms = R->ready_ms, st->finish_ms = R->finish_ms;
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
	return err ? set_error(err, err == NLC_EBLOWUP    ? "non-finite entropy"
	                            : err == NLC_ETIMEDOUT ? "a bounded wait of the tensor-core projection ran out"
	                                                   : "request failed")
	           : NLC_OK;
}
