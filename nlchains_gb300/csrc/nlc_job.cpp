// Level-2 (jobs) and level-3 (the reference command line) of the C ABI.
#include <chrono>
#include <cmath>
#include <csignal>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <thread>

#include "nlc_host.h"

using namespace nlc;

// ------------------------------------------------------------------------------------------------
// jobs
// ------------------------------------------------------------------------------------------------

struct Job {
	nlc_plan *plan = nullptr;
	nlc_model model{};
	uint32_t batching = 1;
	double2 *d_state = nullptr;
	double *d_diag = nullptr;   // [n] linenergies + [2] entropies
	double *h_diag = nullptr;   // pinned copy
	cudaStream_t stream = nullptr;
	size_t state_bytes = 0;
	// pipelined sampling: two result slots (device diagnostics, pinned copies, optional pinned state)
	double *d_slot[2] = {nullptr, nullptr}, *h_slot[2] = {nullptr, nullptr};
	double2 *h_state_slot[2] = {nullptr, nullptr};
	cudaEvent_t ev_slot[2] = {nullptr, nullptr};
	bool slot_state[2] = {false, false};
	cudaEvent_t ev_order = nullptr;   // marks the end of the queued work for jobs ordered after this one
	// one batch + its sample as a CUDA graph, per [slot][copy_state], captured on first use
	cudaGraphExec_t step_exec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
	uint64_t step_kernels[2][2] = {{0, 0}, {0, 0}};

	~Job() {
		if (stream) cudaStreamSynchronize(stream);
		for (auto &row : step_exec)
			for (cudaGraphExec_t g : row)
				if (g) cudaGraphExecDestroy(g);
		if (plan) nlc_plan_destroy(plan);
		cudaFree(d_state);
		cudaFree(d_diag);
		cudaFreeHost(h_diag);
		for (int i = 0; i < 2; i++) {
			cudaFree(d_slot[i]);
			cudaFreeHost(h_slot[i]);
			cudaFreeHost(h_state_slot[i]);
			if (ev_slot[i]) cudaEventDestroy(ev_slot[i]);
		}
		if (ev_order) cudaEventDestroy(ev_order);
		if (stream) cudaStreamDestroy(stream);
	}
};

struct nlc_ctx {
	int device = 0;
	uint64_t next_id = 1;
	std::map<uint64_t, std::unique_ptr<Job>> jobs;
};

static Job *find_job(nlc_ctx *ctx, uint64_t id) {
	if (!ctx) return nullptr;
	auto it = ctx->jobs.find(id);
	return it == ctx->jobs.end() ? nullptr : it->second.get();
}

extern "C" int nlc_create(nlc_ctx **out, int device) {
	if (!out) return set_error(NLC_EINVAL, "ctx pointer is NULL");
	int count = 0;
	int rc = cuda_status(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
	if (rc) return rc;
	if (device < 0 || device >= count) return set_error(NLC_EINVAL, "no such CUDA device");
	auto *c = new nlc_ctx;
	c->device = device;
	*out = c;
	return NLC_OK;
}

extern "C" int nlc_destroy(nlc_ctx *ctx) {
	if (!ctx) return NLC_OK;
	{
		DeviceScope ds(ctx->device);
		ctx->jobs.clear();
	}
	delete ctx;
	return NLC_OK;
}

extern "C" int nlc_job_create(nlc_ctx *ctx, const nlc_model *model, uint32_t batching, uint64_t *id) {
	if (!ctx || !model || !id) return set_error(NLC_EINVAL, "NULL argument");
	if (!batching) return set_error(NLC_EINVAL, "--kernel_batching must be a positive number");
	DeviceScope ds(ctx->device);
	int rc;
	std::unique_ptr<Job> J(new Job);
	J->model = *model;
	J->batching = batching;
	if ((rc = nlc_plan_create(model, &J->plan))) return rc;
	J->model.masses = nullptr;
	J->model.entropy_mask = nullptr;
	const size_t n = model->chain_length;
	J->state_bytes = n * model->copies * sizeof(double2);
	if ((rc = cuda_status(cudaStreamCreateWithFlags(&J->stream, cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
	if ((rc = cuda_status(cudaMalloc(&J->d_state, J->state_bytes), "cudaMalloc state"))) return rc;
	if ((rc = cuda_status(cudaMalloc(&J->d_diag, (n + 2) * sizeof(double)), "cudaMalloc"))) return rc;
	if ((rc = cuda_status(cudaMallocHost(&J->h_diag, (n + 2) * sizeof(double)), "cudaMallocHost"))) return rc;
	*id = ctx->next_id++;
	ctx->jobs[*id] = std::move(J);
	return NLC_OK;
}

extern "C" int nlc_job_destroy(nlc_ctx *ctx, uint64_t id) {
	DeviceScope ds(ctx ? ctx->device : -1);
	if (!find_job(ctx, id)) return set_error(NLC_ENOTFOUND, "no such job");
	ctx->jobs.erase(id);
	return NLC_OK;
}

extern "C" int nlc_job_upload(nlc_ctx *ctx, uint64_t id, const void *host) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	if (!host) return set_error(NLC_EINVAL, "host state is NULL");
	return cuda_status(cudaMemcpyAsync(J->d_state, host, J->state_bytes, cudaMemcpyHostToDevice, J->stream), "upload");
}

extern "C" int nlc_job_download(nlc_ctx *ctx, uint64_t id, void *host) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	if (!host) return set_error(NLC_EINVAL, "host state is NULL");
	int rc = cuda_status(cudaMemcpyAsync(host, J->d_state, J->state_bytes, cudaMemcpyDeviceToHost, J->stream), "download");
	if (rc) return rc;
	return cuda_status(cudaStreamSynchronize(J->stream), "download");
}

extern "C" int nlc_job_advance(nlc_ctx *ctx, uint64_t id, uint64_t steps) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	if (steps % J->batching) return set_error(NLC_EINVAL, "--steps must be a multiple of --kernel_batching");
	// one round of kernel_batching steps per reference launch; rounds with no sample in between may
	// share a launch (move_rounds: the same operations, fewer launches for small ensembles)
	return move_rounds(J->plan, J->d_state, steps / J->batching, J->batching, J->stream);
}

extern "C" int nlc_job_linenergies(nlc_ctx *ctx, uint64_t id, double *lin, double *wt, double *inf) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	const size_t n = J->model.chain_length;
	int rc = nlc_linenergies(J->plan, J->d_state, J->d_diag, J->d_diag + n, J->stream);
	if (rc) return rc;
	if ((rc = cuda_status(cudaMemcpyAsync(J->h_diag, J->d_diag, (n + 2) * sizeof(double), cudaMemcpyDeviceToHost,
	                                      J->stream),
	                      "diagnostics copy")))
		return rc;
	if ((rc = cuda_status(cudaStreamSynchronize(J->stream), "diagnostics"))) return rc;
	if (lin) std::memcpy(lin, J->h_diag, n * sizeof(double));
	if (wt) *wt = J->h_diag[n];
	if (inf) *inf = J->h_diag[n + 1];
	if (!std::isfinite(J->h_diag[n]) || !std::isfinite(J->h_diag[n + 1])) {
		if ((rc = plan_device_status(J->plan))) return rc;
		return set_error(NLC_EBLOWUP, "non-finite entropy (blow-up or vanishing mode energy)");
	}
	return NLC_OK;
}

extern "C" int nlc_job_energies(nlc_ctx *ctx, uint64_t id, double *host_energies) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	if (!host_energies) return set_error(NLC_EINVAL, "NULL argument");
	double *d = nullptr;
	const size_t bytes = size_t(J->model.copies) * sizeof(double);
	int rc = cuda_status(cudaMallocAsync(reinterpret_cast<void **>(&d), bytes, J->stream), "cudaMallocAsync");
	if (rc) return rc;
	rc = nlc_energies(J->plan, J->d_state, d, J->stream);
	if (!rc) rc = cuda_status(cudaMemcpyAsync(host_energies, d, bytes, cudaMemcpyDeviceToHost, J->stream), "energies copy");
	cudaFreeAsync(d, J->stream);
	const int rs = cuda_status(cudaStreamSynchronize(J->stream), "energies");
	return rc ? rc : rs;
}

namespace {

// the result slot's buffers and event, allocated on first use
int ensure_slot(Job *J, int slot, int copy_state) {
	const size_t n = J->model.chain_length;
	int rc;
	if (!J->d_slot[slot]) {
		if ((rc = cuda_status(cudaMalloc(&J->d_slot[slot], (n + 2) * sizeof(double)), "cudaMalloc"))) return rc;
		if ((rc = cuda_status(cudaMallocHost(&J->h_slot[slot], (n + 2) * sizeof(double)), "cudaMallocHost"))) return rc;
		if ((rc = cuda_status(cudaEventCreateWithFlags(&J->ev_slot[slot], cudaEventDisableTiming), "cudaEventCreate")))
			return rc;
	}
	if (copy_state && !J->h_state_slot[slot] &&
	    (rc = cuda_status(cudaMallocHost(&J->h_state_slot[slot], J->state_bytes), "cudaMallocHost")))
		return rc;
	return NLC_OK;
}

// diagnostics of the current state into the slot, the read-backs and the slot's event; `external`
// records the event as an event node of a graph being captured
int enqueue_sample(Job *J, int slot, int copy_state, bool external) {
	const size_t n = J->model.chain_length;
	int rc;
	if ((rc = nlc_linenergies(J->plan, J->d_state, J->d_slot[slot], J->d_slot[slot] + n, J->stream))) return rc;
	if ((rc = cuda_status(cudaMemcpyAsync(J->h_slot[slot], J->d_slot[slot], (n + 2) * sizeof(double),
	                                      cudaMemcpyDeviceToHost, J->stream),
	                      "diagnostics copy")))
		return rc;
	if (copy_state &&
	    (rc = cuda_status(cudaMemcpyAsync(J->h_state_slot[slot], J->d_state, J->state_bytes, cudaMemcpyDeviceToHost,
	                                      J->stream),
	                      "state copy")))
		return rc;
	return cuda_status(cudaEventRecordWithFlags(J->ev_slot[slot], J->stream, external ? cudaEventRecordExternal : 0),
	                   "cudaEventRecord");
}

}  // namespace

extern "C" int nlc_job_sample_async(nlc_ctx *ctx, uint64_t id, int32_t slot, int32_t copy_state) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	if (slot < 0 || slot > 1) return set_error(NLC_EINVAL, "slot must be 0 or 1");
	int rc = ensure_slot(J, slot, copy_state);
	if (rc) return rc;
	if ((rc = enqueue_sample(J, slot, copy_state, false))) return rc;
	J->slot_state[slot] = copy_state != 0;
	return NLC_OK;
}

extern "C" int nlc_job_step_async(nlc_ctx *ctx, uint64_t id, int32_t slot, int32_t copy_state) {
	DeviceScope ds(ctx ? ctx->device : -1);
	NvtxRange r("nlc_job_step");
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	if (slot < 0 || slot > 1) return set_error(NLC_EINVAL, "slot must be 0 or 1");
	int rc = ensure_slot(J, slot, copy_state);
	if (rc) return rc;
	const int cs = copy_state ? 1 : 0;
	if (!J->step_exec[slot][cs]) {
		// capture the batch (its fused launches) and the sample once; the graph replays them with one
		// launch per batch.  Nothing in them allocates or synchronises.
		const uint64_t k0 = launch_count();
		if ((rc = cuda_status(cudaStreamBeginCapture(J->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture")))
			return rc;
		rc = nlc_move(J->plan, J->d_state, J->batching, J->stream);
		if (!rc) rc = enqueue_sample(J, slot, copy_state, true);
		cudaGraph_t g = nullptr;
		const cudaError_t e = cudaStreamEndCapture(J->stream, &g);
		const uint64_t kernels = launch_count() - k0;
		uncount_launch(kernels);
		if (!rc && e != cudaSuccess) rc = cuda_status(e, "cudaStreamEndCapture");
		if (!rc) rc = cuda_status(cudaGraphInstantiate(&J->step_exec[slot][cs], g, 0), "cudaGraphInstantiate");
		if (g) cudaGraphDestroy(g);
		if (rc) return rc;
		J->step_kernels[slot][cs] = kernels;
	}
	J->slot_state[slot] = copy_state != 0;
	count_launch(J->step_kernels[slot][cs]);
	return cuda_status(cudaGraphLaunch(J->step_exec[slot][cs], J->stream), "cudaGraphLaunch");
}

extern "C" int nlc_job_sample_wait(nlc_ctx *ctx, uint64_t id, int32_t slot, double *lin, double *wt, double *inf,
                                   void *host_state, int32_t timeout_ms) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	if (slot < 0 || slot > 1 || !J->ev_slot[slot]) return set_error(NLC_EINVAL, "slot was never filled");
	if (host_state && !J->slot_state[slot]) return set_error(NLC_EINVAL, "slot holds no state copy");
	const auto t0 = std::chrono::steady_clock::now();
	for (;;) {
		const cudaError_t e = cudaEventQuery(J->ev_slot[slot]);
		if (e == cudaSuccess) break;
		if (e != cudaErrorNotReady) return cuda_status(e, "sample");
		const auto waited = std::chrono::steady_clock::now() - t0;
		if (timeout_ms >= 0 && waited >= std::chrono::milliseconds(timeout_ms))
			return set_error(NLC_ETIMEDOUT, "sample not ready");
		// poll for the first half millisecond (short batches), then yield the core in short naps
		if (waited >= std::chrono::microseconds(500)) std::this_thread::sleep_for(std::chrono::microseconds(20));
	}
	const size_t n = J->model.chain_length;
	const double *h = J->h_slot[slot];
	if (lin) std::memcpy(lin, h, n * sizeof(double));
	if (wt) *wt = h[n];
	if (inf) *inf = h[n + 1];
	if (host_state) std::memcpy(host_state, J->h_state_slot[slot], J->state_bytes);
	if (!std::isfinite(h[n]) || !std::isfinite(h[n + 1])) {
		if (const int rc = plan_device_status(J->plan)) return rc;
		return set_error(NLC_EBLOWUP, "non-finite entropy (blow-up or vanishing mode energy)");
	}
	return NLC_OK;
}

extern "C" int nlc_job_after(nlc_ctx *ctx, uint64_t id, uint64_t after_id) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	Job *A = find_job(ctx, after_id);
	if (!J || !A) return set_error(NLC_ENOTFOUND, "no such job");
	if (J == A) return NLC_OK;   // a job's own work is in order already
	int rc;
	if (!A->ev_order &&
	    (rc = cuda_status(cudaEventCreateWithFlags(&A->ev_order, cudaEventDisableTiming), "cudaEventCreate")))
		return rc;
	if ((rc = cuda_status(cudaEventRecord(A->ev_order, A->stream), "cudaEventRecord"))) return rc;
	return cuda_status(cudaStreamWaitEvent(J->stream, A->ev_order, 0), "cudaStreamWaitEvent");
}

extern "C" int nlc_job_wait(nlc_ctx *ctx, uint64_t id, int32_t timeout_ms) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	const auto t0 = std::chrono::steady_clock::now();
	for (;;) {
		const cudaError_t e = cudaStreamQuery(J->stream);
		if (e == cudaSuccess) return NLC_OK;
		if (e != cudaErrorNotReady) return cuda_status(e, "job");
		if (timeout_ms >= 0 &&
		    std::chrono::steady_clock::now() - t0 >= std::chrono::milliseconds(timeout_ms))
			return set_error(NLC_ETIMEDOUT, "job still running");
		std::this_thread::sleep_for(std::chrono::microseconds(200));
	}
}

extern "C" int nlc_job_state_ptr(nlc_ctx *ctx, uint64_t id, void **ptr) {
	DeviceScope ds(ctx ? ctx->device : -1);
	Job *J = find_job(ctx, id);
	if (!J) return set_error(NLC_ENOTFOUND, "no such job");
	if (!ptr) return set_error(NLC_EINVAL, "NULL argument");
	*ptr = J->d_state;
	return NLC_OK;
}

// ------------------------------------------------------------------------------------------------
// the reference command line (common/main.cpp, common/configuration.hpp, common/results.cpp)
// ------------------------------------------------------------------------------------------------

namespace {

volatile std::sig_atomic_t g_quit = 0;

struct Opt {
	const char *lng;   // long name
	char shrt;         // short name or 0
	bool value;        // takes a value
	const char *help;
};

const Opt kCommon[] = {
	{"verbose", 'v', false, "print extra informations"},
	{"initial", 'i', true, "initial state file"},
	{"chain_length", 'n', true, "length of the chain"},
	{"copies", 'c', true, "number of realizations of the chain in the ensemble"},
	{"dt", 0, true, "time step value"},
	{"kernel_batching", 'b', true, "number of steps per kernel invocation"},
	{"steps", 's', true, "number of steps in total (0 for infinite)"},
	{"time_offset", 'o', true, "time offset in dump files"},
	{"entropy", 'e', true, "entropy limit"},
	{"WTlimit", 0, false, "limit WT entropy instead of information entropy"},
	{"entropymask", 0, true, "mask of linenergies to include in entropy calculation"},
	{"prefix", 'p', true, "prefix for dump files"},
	{"dump_interval", 0, true,
	 "number of steps between full state dumps (defaults to same value as --batch, does not affect time granularity of entropy)"},
};

struct CliError {
	int kind;   // 0 invalid argument, 1 I/O
	std::string msg;
};

std::vector<Opt> model_options(const std::string &prog) {
	std::vector<Opt> o;
	if (prog == "DNKG") {
		o.push_back({"m", 'm', true, "linear parameter m"});
		o.push_back({"beta", 0, true, "fourth order nonlinearity"});
	} else if (prog == "FPUT") {
		o.push_back({"alpha", 0, true, "third order nonlinearity"});
		o.push_back({"beta", 0, true, "fourth order nonlinearity"});
	} else if (prog == "Toda") {
		o.push_back({"alpha", 0, true, "steepness of exponential, V(dx)=e^(2*alpha*dx)/(4*alpha^2)-dx/(2*alpha)"});
	} else if (prog == "dDNKG") {
		o.push_back({"m", 'm', true, "linear parameter m filename"});
		o.push_back({"beta", 0, true, "fourth order nonlinearity"});
	} else if (prog == "DNLS") {
		o.push_back({"no_linear_callback", 0, false, "do not use cuFFT callback for linear evolution (accepted, no effect)"});
		o.push_back({"no_nonlinear_callback", 0, false, "do not use cuFFT callback for nonlinear evolution (accepted, no effect)"});
		o.push_back({"beta", 0, true, "fourth order nonlinearity"});
	}
	if (prog != "DNLS") o.push_back({"split_kernel", 0, false, "force use of split kernel"});
	return o;
}

std::string usage(const std::string &prog, const std::vector<Opt> &opts) {
	std::ostringstream s;
	s << "Options for " << prog << ":\n";
	for (const Opt &o : opts) {
		std::string name = o.shrt && std::string(o.lng) != std::string(1, o.shrt) ? std::string("-") + o.shrt + " [ --" + o.lng + " ]"
		                   : o.shrt                                            ? std::string("-") + o.shrt
		                                                                       : std::string("--") + o.lng;
		if (o.value) name += " arg";
		s << "  " << name;
		for (size_t i = name.size(); i < 30; i++) s << ' ';
		s << o.help << "\n";
	}
	return s.str();
}

// Boost.Program_options-style parsing: -x v, -xv, --name v, --name=v, unique long-name prefixes.
std::map<std::string, std::string> parse(int argc, char **argv, const std::vector<Opt> &opts) {
	std::map<std::string, std::string> vm;
	for (int i = 1; i < argc; i++) {
		std::string a = argv[i];
		const Opt *o = nullptr;
		std::string val;
		bool has_val = false;
		if (a.size() > 2 && a[0] == '-' && a[1] == '-') {
			std::string name = a.substr(2);
			const size_t eq = name.find('=');
			if (eq != std::string::npos) val = name.substr(eq + 1), name = name.substr(0, eq), has_val = true;
			std::vector<const Opt *> hits;
			for (const Opt &c : opts) {
				if (name == c.lng) {
					hits.assign(1, &c);
					break;
				}
				if (std::string(c.lng).compare(0, name.size(), name) == 0) hits.push_back(&c);
			}
			if (hits.size() != 1)
				throw CliError{0, (hits.empty() ? "unrecognised option '" : "option '") + a +
				                      (hits.empty() ? "'" : "' is ambiguous")};
			o = hits[0];
		} else if (a.size() >= 2 && a[0] == '-') {
			for (const Opt &c : opts)
				if (c.shrt == a[1]) o = &c;
			if (!o) throw CliError{0, "unrecognised option '" + a + "'"};
			if (a.size() > 2) val = a.substr(2), has_val = true;
		} else {
			throw CliError{0, "unexpected positional argument '" + a + "'"};
		}
		if (o->value) {
			if (!has_val) {
				if (i + 1 >= argc) throw CliError{0, std::string("the required argument for option '--") + o->lng + "' is missing"};
				val = argv[++i];
			}
		} else if (has_val) {
			throw CliError{0, std::string("option '--") + o->lng + "' does not take any arguments"};
		}
		if (vm.count(o->lng)) throw CliError{0, std::string("option '--") + o->lng + "' cannot be specified more than once"};
		vm[o->lng] = val;
	}
	return vm;
}

template <typename T>
T num(const std::map<std::string, std::string> &vm, const char *name, T dflt, bool required) {
	auto it = vm.find(name);
	if (it == vm.end()) {
		if (required) throw CliError{0, std::string("the option '--") + name + "' is required but missing"};
		return dflt;
	}
	std::istringstream s(it->second);
	T v{};
	s >> v;
	if (s.fail() || !s.eof()) throw CliError{0, std::string("the argument ('") + it->second + "') for option '--" + name + "' is invalid"};
	if (std::is_unsigned<T>::value && it->second.find('-') != std::string::npos)
		throw CliError{0, std::string("the argument ('") + it->second + "') for option '--" + name + "' is invalid"};
	return v;
}

std::vector<char> read_file(const std::string &path, size_t bytes, const char *what) {
	std::ifstream f(path, std::ios::binary);
	std::vector<char> buf(bytes);
	if (!f || !f.read(buf.data(), std::streamsize(bytes)))
		throw CliError{1, std::string("could not read ") + what + " (" + path + ")"};
	return buf;
}

void write_file(const std::string &path, const void *data, size_t bytes, const char *what) {
	std::ofstream f(path, std::ios::binary | std::ios::trunc);
	if (!f || !f.write(static_cast<const char *>(data), std::streamsize(bytes)))
		throw CliError{1, std::string("cannot open ") + what + " file (" + path + ")"};
}

int run_program(int argc, char **argv) {
	const std::string prog = argv[0];
	static const char *kPrograms[] = {"DNKG", "FPUT", "Toda", "dDNKG", "DNLS"};
	bool known = false;
	for (const char *p : kPrograms) known |= prog == p;
	if (!known) {
		if (prog.size() > 4 && prog.compare(prog.size() - 4, 4, "-cpu") == 0)
			throw CliError{0, "the CPU validation subprograms are not part of this engine; run " + prog.substr(0, prog.size() - 4)};
		throw CliError{0, "please specific a valid program among DNKG, DNLS, FPUT, Toda, dDNKG"};
	}
	std::vector<Opt> opts(std::begin(kCommon), std::end(kCommon));
	for (const Opt &o : model_options(prog)) opts.push_back(o);
	if (argc == 1) {
		std::cout << usage(prog, opts);
		return 0;
	}
	std::map<std::string, std::string> vm;
	try {
		vm = parse(argc, argv, opts);
	} catch (CliError &e) {
		e.msg += "\n" + usage(prog, opts);
		throw;
	}
	const bool verbose = vm.count("verbose");
	nlc_model M{};
	const std::string initial = vm.count("initial") ? vm["initial"] : "";
	M.chain_length = num<uint32_t>(vm, "chain_length", 0, true);
	M.copies = num<uint32_t>(vm, "copies", 0, true);
	M.dt = num<double>(vm, "dt", 0, true);
	const uint32_t batching = num<uint32_t>(vm, "kernel_batching", 0, true);
	const uint64_t steps = num<uint64_t>(vm, "steps", 0, false);
	const uint64_t offset = num<uint64_t>(vm, "time_offset", 0, false);
	const std::string prefix = vm.count("prefix") ? vm["prefix"] : "";
	if (!vm.count("initial")) throw CliError{0, "the option '--initial' is required but missing\n" + usage(prog, opts)};
	if (!vm.count("prefix")) throw CliError{0, "the option '--prefix' is required but missing\n" + usage(prog, opts)};
	const bool has_entropy = vm.count("entropy");
	const double entropy_limit = num<double>(vm, "entropy", 0, false);
	const bool wt_limit = vm.count("WTlimit");
	uint32_t dump_interval = batching;
	// main.cpp:82-103
	if (M.chain_length < 2 || !M.copies || !(M.dt > 0) || !batching)
		throw CliError{0, "--chain_length must be >= 2, --copies, --dt and --kernel_batching must be positive numbers\n" + usage(prog, opts)};
	if (M.chain_length > 65535) throw CliError{0, "--chain_length must fit 16 bits\n" + usage(prog, opts)};
	if (vm.count("dump_interval")) {
		dump_interval = num<uint32_t>(vm, "dump_interval", 0, false);
		if (!dump_interval) throw CliError{0, "--dump_interval must be > 0\n" + usage(prog, opts)};
	}
	if (prefix.empty()) throw CliError{0, "--prefix must not be an empty string\n" + usage(prog, opts)};
	if (dump_interval % batching) throw CliError{0, "--dump_interval must be a multiple of --kernel_batching\n" + usage(prog, opts)};
	if (steps % batching) throw CliError{0, "--steps must be a multiple of --kernel_batching\n" + usage(prog, opts)};
	if (offset && steps && offset >= steps) throw CliError{0, "--time_offset must be less than --steps\n" + usage(prog, opts)};

	std::vector<double> masses;
	if (prog == "DNKG") M.model = NLC_DNKG, M.m = num<double>(vm, "m", 0, true), M.beta = num<double>(vm, "beta", 0, true);
	if (prog == "FPUT") M.model = NLC_FPUT, M.alpha = num<double>(vm, "alpha", 0, true), M.beta = num<double>(vm, "beta", 0, true);
	if (prog == "Toda") M.model = NLC_TODA, M.alpha = num<double>(vm, "alpha", 0, true);
	if (prog == "DNLS") M.model = NLC_DNLS, M.beta = num<double>(vm, "beta", 0, true);
	if (prog == "dDNKG") {
		M.model = NLC_DDNKG;
		M.beta = num<double>(vm, "beta", 0, true);
		if (!vm.count("m")) throw CliError{0, "the option '-m' is required but missing\n" + usage(prog, opts)};
		auto raw = read_file(vm["m"], M.chain_length * sizeof(double), "m file");
		masses.resize(M.chain_length);
		std::memcpy(masses.data(), raw.data(), raw.size());
		M.masses = masses.data();
	}
	if (vm.count("split_kernel")) M.flags |= NLC_FLAG_SPLIT_KERNEL;
	std::vector<uint8_t> mask;
	if (vm.count("entropymask")) {
		auto raw = read_file(vm["entropymask"], M.chain_length, "entropy mask file");
		mask.assign(raw.begin(), raw.end());
		size_t used = 0;
		for (uint8_t b : mask) used += b != 0;
		if (used < 2) throw CliError{0, "Too few modes for entropy calculation\n" + usage(prog, opts)};
		M.entropy_mask = mask.data();
	}
	const size_t n = M.chain_length, state_bytes = n * M.copies * sizeof(double2);
	// main.cpp:112-118: the initial state is read before any device work
	std::vector<double> host(2 * n * M.copies);
	double *host_state = host.data();
	{
		std::ifstream f(initial, std::ios::binary);
		if (!f || !f.read(reinterpret_cast<char *>(host_state), std::streamsize(state_bytes)))
			throw CliError{1, "could not read initial state (" + initial + ")"};
	}

	nlc_ctx *ctx = nullptr;
	if (nlc_create(&ctx, 0)) throw CliError{2, nlc_last_error()};
	std::unique_ptr<nlc_ctx, int (*)(nlc_ctx *)> ctx_guard(ctx, nlc_destroy);
	uint64_t job = 0;
	int rc = nlc_job_create(ctx, &M, batching, &job);
	if (rc) throw CliError{rc == NLC_EINVAL ? 0 : 2, nlc_last_error()};
	if (verbose) {
		int32_t lanes, sites, threads, tier;
		nlc_plan_shape(find_job(ctx, job)->plan, &lanes, &sites, &threads, &tier);
		cudaDeviceProp p{};
		cudaGetDeviceProperties(&p, ctx->device);
		std::cout << "nlchains-gb300: GPU " << p.name << ", integrator tier " << tier << ", " << lanes
		          << " lanes/chain, " << sites << " sites/lane, " << threads << " threads/block" << std::endl;
	}
	if (M.model == NLC_DDNKG) {
		// eigensystem.cpp:23-29: -omegas (n doubles), -eigenvectors (n x n, column-major)
		std::vector<double> om(n);
		nlc_plan_omegas(find_job(ctx, job)->plan, om.data());
		write_file(prefix + "-omegas", om.data(), n * sizeof(double), "eigensystem");
		// the eigenvectors the plan's projection uses
		const std::vector<double> *vec = plan_eigenvectors(find_job(ctx, job)->plan);
		if (!vec) throw CliError{2, "no eigensystem in the dDNKG plan"};
		write_file(prefix + "-eigenvectors", vec->data(), vec->size() * sizeof(double), "eigensystem");
	}
	if ((rc = nlc_job_upload(ctx, job, host_state))) throw CliError{2, nlc_last_error()};

	std::ofstream entropy_file(prefix + "-entropy", std::ios::binary | std::ios::trunc);
	if (!entropy_file) throw CliError{1, "cannot open entropy file (" + prefix + "-entropy)"};
	std::vector<double> lin(n);
	auto dump = [&](uint64_t t, bool state) {
		write_file(prefix + "-linenergies-" + std::to_string(t), lin.data(), n * sizeof(double), "linenergies");
		if (state) {
			if (nlc_job_download(ctx, job, host_state)) throw CliError{2, nlc_last_error()};
			write_file(prefix + "-" + std::to_string(t), host_state, state_bytes, "dump");
		}
	};
	// Pipelined like the reference's loop (DNKG_FPUT_Toda.cpp:108-151, loop_control.hpp): the next
	// batch and its sample are enqueued before the host handles the current sample (entropy line,
	// limit checks, dumps), so the GPU integrates while the files are written.  A quit request (signal,
	// entropy limit, non-finite entropy: results.cpp:63-73) stops the loop at the step of the sample
	// already in flight, within the reference's own range (it stops at its main loop's step, up to
	// two batches past the sample that asked).
	uint64_t t = offset;
	int slot = 0;
	if ((rc = nlc_job_sample_async(ctx, job, slot, t % dump_interval == 0))) throw CliError{2, nlc_last_error()};
	bool quit = false, in_flight = false;
	for (;;) {
		const bool last = (steps && t == steps) || quit;
		in_flight = false;
		if (!last) {
			// the next batch and its sample: one graph launch
			const uint64_t tn = t + batching;
			if ((rc = nlc_job_step_async(ctx, job, slot ^ 1, tn % dump_interval == 0))) throw CliError{2, nlc_last_error()};
			in_flight = true;
		}
		double wt = 0, inf = 0;
		const bool full_dump = t % dump_interval == 0;
		rc = nlc_job_sample_wait(ctx, job, slot, lin.data(), &wt, &inf, full_dump ? host_state : nullptr, -1);
		if (rc == NLC_EBLOWUP) quit = true;   // results.cpp:64-68
		else if (rc) throw CliError{2, nlc_last_error()};
		if (g_quit) quit = true;
		const double triplet[3] = {t * M.dt, wt, inf};
		entropy_file.write(reinterpret_cast<const char *>(triplet), sizeof(triplet)).flush();
		if (verbose) std::cout << "Entropy step " << t << ": " << wt << '/' << inf << std::endl;
		if (has_entropy && (wt_limit ? wt : inf) < entropy_limit) quit = true;   // results.cpp:69-72
		if (full_dump) {
			write_file(prefix + "-linenergies-" + std::to_string(t), lin.data(), n * sizeof(double), "linenergies");
			write_file(prefix + "-" + std::to_string(t), host_state, state_bytes, "dump");
		}
		if (!in_flight) break;   // after a quit request the sample in flight is handled, then the loop stops
		t += batching;
		slot ^= 1;
	}
	if (t % dump_interval != 0) dump(t, true);
	return 0;
}

}  // namespace

extern "C" int nlc_program_run(int argc, char **argv) {
	if (argc < 1 || !argv || !argv[0]) {
		std::cout << "Please specify as first argument the subprogram to run: DNKG, DNLS, FPUT, Toda, dDNKG" << std::endl;
		return 0;
	}
	g_quit = 0;
	auto prev_int = std::signal(SIGINT, [](int) { g_quit = 1; });
	auto prev_term = std::signal(SIGTERM, [](int) { g_quit = 1; });
	int ret = 0;
	try {
		ret = run_program(argc, argv);
	} catch (const CliError &e) {
		const char *kind = e.kind == 0 ? "invalid argument, " : e.kind == 1 ? "I/O error, " : "";
		std::cerr << "nlchains: " << kind << e.msg << std::endl;
		set_error(e.kind == 0 ? NLC_EINVAL : e.kind == 1 ? NLC_EIO : NLC_ECUDA, e.msg);
		ret = 1;
	} catch (const std::exception &e) {
		std::cerr << "nlchains: exception, " << e.what() << std::endl;
		ret = 1;
	}
	std::signal(SIGINT, prev_int);
	std::signal(SIGTERM, prev_term);
	return ret;
}

// Host entropies of the linear energies e over the selected modes M (|M| = count):
// e' = e |M| / sum e, WT = -sum log e', INF = sum e' log e' (results_entropy.cpp:21-46), written
// with the normalisation taken out of the sums: WT = -(sum log e + |M| log r), INF =
// r (sum e log e + log r sum e), r = |M| / sum e.
extern "C" int nlc_entropies(const double *lin, uint32_t n, int32_t a0is0, const uint8_t *mask, double *out) {
	if (!lin || !out) return set_error(NLC_EINVAL, "nlc_entropies: NULL argument");
	double sum_e = 0, sum_log = 0, sum_elog = 0;
	uint32_t count = 0;
	for (uint32_t k = 0; k < n; k++) {
		if ((mask && !mask[k]) || (a0is0 && k == 0)) continue;
		const double lk = std::log(lin[k]);
		sum_e += lin[k];
		sum_log += lk;
		sum_elog += lin[k] * lk;
		count++;
	}
	if (!count) return set_error(NLC_EINVAL, "nlc_entropies: no mode selected");
	const double r = count / sum_e, lr = std::log(r);
	out[0] = -(sum_log + count * lr);
	out[1] = r * (sum_elog + lr * sum_e);
	if (!std::isfinite(out[0]) || !std::isfinite(out[1]))
		return set_error(NLC_EBLOWUP, "non-finite entropy");
	return NLC_OK;
}
