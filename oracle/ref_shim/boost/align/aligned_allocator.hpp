/*
 * TEST INFRASTRUCTURE ONLY -- stand-in for boost::alignment::aligned_allocator<T, A>, the
 * allocator behind the reference's simd_allocator (common/utilities.hpp:186).
 */
#pragma once

#include <cstddef>
#include <cstdlib>
#include <new>

namespace boost {
namespace alignment {

template<typename T, std::size_t Alignment>
struct aligned_allocator {
	typedef T value_type;

	template<typename U>
	struct rebind {
		typedef aligned_allocator<U, Alignment> other;
	};

	aligned_allocator() = default;

	template<typename U>
	aligned_allocator(const aligned_allocator<U, Alignment> &) {}

	T *allocate(std::size_t n) {
		void *p = nullptr;
		std::size_t a = Alignment < alignof(T) ? alignof(T) : Alignment;
		if (posix_memalign(&p, a, n * sizeof(T) ? n * sizeof(T) : a)) throw std::bad_alloc();
		return static_cast<T *>(p);
	}

	void deallocate(T *p, std::size_t) { std::free(p); }

	template<typename U>
	bool operator==(const aligned_allocator<U, Alignment> &) const { return true; }

	template<typename U>
	bool operator!=(const aligned_allocator<U, Alignment> &) const { return false; }
};

}  // namespace alignment
}  // namespace boost
