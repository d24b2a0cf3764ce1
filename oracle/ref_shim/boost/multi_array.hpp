/*
 * TEST INFRASTRUCTURE ONLY -- stand-in for the two-dimensional boost::multi_array that holds the
 * reference's DNLS linear-propagator tables (DNLS/dispersion.cpp:19-26, DNLS/cpu-implementation/
 * DNLS.cpp:39-44): construction from extents[a][b], row indexing, row iteration.
 */
#pragma once

#include <cstddef>
#include <vector>

namespace boost {

namespace detail_shim {
struct extent_2 {
	std::size_t rows, cols;
};

struct extent_1 {
	std::size_t rows;

	extent_2 operator[](std::size_t cols) const { return {rows, cols}; }
};

struct extent_gen {
	extent_1 operator[](std::size_t rows) const { return {rows}; }
};
}  // namespace detail_shim

static const detail_shim::extent_gen extents{};

template<typename T, std::size_t Dims>
struct multi_array;

template<typename T>
struct multi_array<T, 2> {
	explicit multi_array(detail_shim::extent_2 e) : cols(e.cols), data(e.rows * e.cols) {}

	struct row {
		T *p;
		std::size_t n;

		T &operator[](std::size_t j) const { return p[j]; }

		T *begin() const { return p; }

		T *end() const { return p + n; }
	};

	row operator[](std::size_t i) { return row{data.data() + i * cols, cols}; }

private:
	std::size_t cols;
	std::vector<T> data;
};

}  // namespace boost
