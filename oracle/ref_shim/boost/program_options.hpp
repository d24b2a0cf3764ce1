/*
 * TEST INFRASTRUCTURE ONLY -- a stand-in for the subset of Boost.ProgramOptions that the
 * reference's command line uses (common/main.cpp:53-70, common/wisdom_sync.hpp:194-198 and the
 * per-model option blocks), so that the reference's own CPU sources compile and run in place for
 * the oracle's parity fixtures.  Written for this repository; not Boost's code.
 *
 * Supported: options_description with add_options() chains, value(&x) with ->required() and
 * ->default_value(v), switches without a value, "long,s" names, "--long value", "--long=value",
 * "-s value" and "-svalue"; store(), notify(), variables_map::count(); errors derive from
 * boost::program_options::error (a std::logic_error) as in Boost.
 */
#pragma once

#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <limits>
#include <map>
#include <memory>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace boost {
namespace program_options {

struct error : std::logic_error {
	explicit error(const std::string &what) : std::logic_error(what) {}
};

struct value_semantic {
	virtual ~value_semantic() = default;
	virtual void parse(const std::string &name, const std::string &text) = 0;
	virtual bool has_default() const = 0;
	virtual void apply_default() = 0;
	virtual bool is_required() const = 0;
};

namespace detail {
template<typename T>
typename std::enable_if<std::is_integral<T>::value, T>::type convert(const std::string &name, const std::string &text) {
	if (text.empty() || text[0] == '-') throw error("the argument ('" + text + "') for option '--" + name + "' is invalid");
	errno = 0;
	char *end = nullptr;
	unsigned long long v = std::strtoull(text.c_str(), &end, 10);
	if (errno || *end || v > std::numeric_limits<T>::max())
		throw error("the argument ('" + text + "') for option '--" + name + "' is invalid");
	return T(v);
}

template<typename T>
typename std::enable_if<std::is_floating_point<T>::value, T>::type convert(const std::string &name, const std::string &text) {
	errno = 0;
	char *end = nullptr;
	double v = std::strtod(text.c_str(), &end);
	if (text.empty() || errno || *end)
		throw error("the argument ('" + text + "') for option '--" + name + "' is invalid");
	return T(v);
}

template<typename T>
typename std::enable_if<std::is_same<T, std::string>::value, T>::type convert(const std::string &, const std::string &text) {
	return text;
}
}  // namespace detail

template<typename T>
struct typed_value : value_semantic {
	explicit typed_value(T *target) : target(target) {}

	typed_value *required() {
		req = true;
		return this;
	}

	typed_value *default_value(const T &v) {
		def = v;
		has_def = true;
		return this;
	}

	void parse(const std::string &name, const std::string &text) override {
		*target = detail::convert<T>(name, text);
	}

	bool has_default() const override { return has_def; }

	void apply_default() override {
		if (has_def) *target = def;
	}

	bool is_required() const override { return req; }

private:
	T *target;
	T def{};
	bool req = false, has_def = false;
};

template<typename T>
typed_value<T> *value(T *target) { return new typed_value<T>(target); }

struct option {
	std::string long_name, short_name, description;
	std::shared_ptr<value_semantic> semantic;   /* null for a switch */

	std::string key() const { return long_name.empty() ? short_name : long_name; }
};

struct options_description {
	explicit options_description(const std::string &caption = "") : caption(caption) {}

	struct easy_init {
		options_description *owner;

		easy_init &operator()(const char *names, value_semantic *semantic, const char *description) {
			owner->add(names, semantic, description);
			return *this;
		}

		easy_init &operator()(const char *names, const char *description) {
			owner->add(names, nullptr, description);
			return *this;
		}
	};

	easy_init add_options() { return easy_init{this}; }

	const option *find_long(const std::string &name) const {
		for (auto &o: opts) if (!o.long_name.empty() && o.long_name == name) return &o;
		return nullptr;
	}

	const option *find_short(const std::string &name) const {
		for (auto &o: opts) if (!o.short_name.empty() && o.short_name == name) return &o;
		return nullptr;
	}

	std::string caption;
	std::vector<option> opts;

private:
	void add(const std::string &names, value_semantic *semantic, const char *description) {
		option o;
		auto comma = names.find(',');
		o.long_name = names.substr(0, comma);
		if (comma != std::string::npos) o.short_name = names.substr(comma + 1);
		o.description = description;
		o.semantic.reset(semantic);
		opts.push_back(std::move(o));
	}
};

inline std::ostream &operator<<(std::ostream &out, const options_description &d) {
	out << d.caption << ":\n";
	for (auto &o: d.opts) {
		out << "  ";
		if (!o.short_name.empty()) out << "-" << o.short_name << (o.long_name.empty() ? "" : " [ --") ;
		else out << "--";
		out << o.long_name;
		if (!o.short_name.empty() && !o.long_name.empty()) out << " ]";
		if (o.semantic) out << " arg";
		out << "\t" << o.description << "\n";
	}
	return out;
}

struct parsed_options {
	const options_description *description = nullptr;
	std::vector<std::pair<const option *, std::string>> items;
};

inline parsed_options parse_command_line(int argc, char *argv[], const options_description &desc) {
	parsed_options parsed;
	parsed.description = &desc;
	for (int i = 1; i < argc; i++) {
		std::string tok = argv[i], name, text;
		bool has_text = false;
		const option *o = nullptr;
		if (tok.size() > 2 && tok[0] == '-' && tok[1] == '-') {
			auto eq = tok.find('=');
			name = tok.substr(2, eq == std::string::npos ? std::string::npos : eq - 2);
			if (eq != std::string::npos) text = tok.substr(eq + 1), has_text = true;
			o = desc.find_long(name);
		} else if (tok.size() > 1 && tok[0] == '-') {
			name = tok.substr(1, 1);
			if (tok.size() > 2) text = tok.substr(2), has_text = true;
			o = desc.find_short(name);
		} else {
			throw error("too many positional options have been specified on the command line");
		}
		if (!o) throw error("unrecognised option '" + tok + "'");
		if (o->semantic) {
			if (!has_text) {
				if (i + 1 >= argc) throw error("the required argument for option '--" + o->key() + "' is missing");
				text = argv[++i];
			}
		} else if (has_text) {
			throw error("option '--" + o->key() + "' does not take any arguments");
		}
		parsed.items.emplace_back(o, text);
	}
	return parsed;
}

struct variables_map {
	size_t count(const std::string &name) const { return seen.count(name); }

	std::map<std::string, std::pair<const option *, std::string>> seen;   /* given on the command line */
	std::map<std::string, const option *> defaulted;
	const options_description *description = nullptr;
};

inline void store(const parsed_options &parsed, variables_map &vm) {
	vm.description = parsed.description;
	for (auto &item: parsed.items) {
		auto key = item.first->key();
		if (vm.seen.count(key)) throw error("option '--" + key + "' cannot be specified more than once");
		vm.seen[key] = item;
	}
	/* Boost counts an option with a default value as present */
	for (auto &o: parsed.description->opts)
		if (o.semantic && o.semantic->has_default() && !vm.seen.count(o.key())) {
			vm.defaulted[o.key()] = &o;
			vm.seen[o.key()] = {&o, std::string()};
		}
}

inline void notify(variables_map &vm) {
	if (!vm.description) return;
	for (auto &o: vm.description->opts)
		if (o.semantic && o.semantic->is_required() && !vm.seen.count(o.key()))
			throw error("the option '--" + o.key() + "' is required but missing");
	for (auto &kv: vm.seen) {
		auto *o = kv.second.first;
		if (!o->semantic) continue;
		if (vm.defaulted.count(kv.first)) o->semantic->apply_default();
		else o->semantic->parse(o->key(), kv.second.second);
	}
}

}  // namespace program_options
}  // namespace boost
