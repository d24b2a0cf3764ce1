/*
 * TEST INFRASTRUCTURE ONLY -- a single-process stand-in for the parts of Boost.MPI and of the MPI C
 * API that the reference's CPU path names (common/main.cpp:17-31, common/mpi_environment.hpp,
 * common/loop_control.hpp:26-37, common/results*.cpp, common/wisdom_sync.hpp,
 * dDNKG/eigensystem.cpp:34-35).  One rank: every collective is the identity, rank 0 of size 1.
 * Written for this repository; not Boost's or any MPI library's code.
 */
#pragma once

#include <cstring>
#include <exception>
#include <string>

typedef int MPI_Comm;
typedef int MPI_Info;
typedef int MPI_Datatype;
typedef int MPI_File;
typedef struct { int unused; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_COMM_TYPE_SHARED 1
#define MPI_INFO_NULL 0
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_DOUBLE 8
#define MPI_STATUS_IGNORE ((MPI_Status *) 0)

/* The node split of a single process is the process itself. */
inline int MPI_Comm_split_type(MPI_Comm, int, int, MPI_Info, MPI_Comm *out) {
	*out = MPI_COMM_WORLD;
	return 0;
}

/* Parallel file output is only reached with more than one rank (results.cpp:104-119). */
inline int MPI_File_open(MPI_Comm, const char *, int, MPI_Info, MPI_File *) { return 1; }
inline int MPI_File_close(MPI_File *) { return 1; }
inline int MPI_File_set_size(MPI_File, long long) { return 1; }
inline int MPI_File_write_ordered(MPI_File, const void *, int, MPI_Datatype, MPI_Status *) { return 1; }

namespace boost {
namespace mpi {

namespace threading {
enum level { single, funneled, serialized, multiple };
}

enum comm_create_kind { comm_duplicate, comm_take_ownership, comm_attach };

struct environment {
	environment(threading::level, bool) {}

	static std::string processor_name() { return "localhost"; }
};

struct communicator {
	communicator() = default;

	communicator(const MPI_Comm &, comm_create_kind) {}

	int rank() const { return 0; }

	int size() const { return 1; }

	operator MPI_Comm() const { return MPI_COMM_WORLD; }
};

template<typename T>
struct maximum {
	T operator()(const T &a, const T &b) const { return a < b ? b : a; }
};

template<typename T, typename Op>
void all_reduce(const communicator &, const T &in, T &out, Op) { out = in; }

template<typename T, typename Op>
void all_reduce(const communicator &, const T *in, int n, T *out, Op) {
	if (in != out) std::memmove(out, in, sizeof(T) * size_t(n));
}

template<typename T>
void broadcast(const communicator &, T &, int) {}

template<typename T>
void broadcast(const communicator &, T *, int, int) {}

struct exception : std::exception {
	exception(const char *routine, int result_code) : routine_(routine), result_code_(result_code),
	                                                   message(std::string(routine) + ": MPI error " +
	                                                           std::to_string(result_code)) {}

	const char *what() const noexcept override { return message.c_str(); }

	int result_code() const { return result_code_; }

protected:
	const char *routine_;
	int result_code_;
	std::string message;
};

}  // namespace mpi
}  // namespace boost
