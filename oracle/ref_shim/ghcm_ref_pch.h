// Force-included prelude that lets the reference's CPU solvers
// (src/eikonal_fim.cpp, src/eikonal_fmm.cpp, src/eikonal.h, src/util_field.h,
// src/util_dim.h, src/bitset_dynamic.h) compile unmodified without their
// third-party submodules, which the reference ships empty (.gitmodules:1-12).
//
// It stands in for the reference's src/pch.h (force-included by
// premake5.lua:25): the standard headers, a minimal glm vector shim (only the
// 2-component types and the relational helpers those files use), std::optional
// in place of akrzemi1/Optional, empty OpenCL handle types (eikonal.h names them
// in prototypes that the CPU solvers never call) and length_of.
//
// TEST INFRASTRUCTURE ONLY: this header builds the checker library
// oracle/_ref/libghcm_ref.so. Nothing in the product links it.
#pragma once

#include <algorithm>
#include <cassert>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <deque>
#include <functional>
#include <iostream>
#include <limits>
#include <optional>
#include <queue>
#include <sstream>
#include <utility>
#include <vector>

namespace glm {

enum precision { highp, mediump, lowp, defaultp = highp };

typedef std::uint8_t  u8;
typedef std::uint32_t u32;

template <typename T, precision P = defaultp>
struct tvec2 {
    T x, y;

    tvec2() : x(0), y(0) {}
    explicit tvec2(T s) : x(s), y(s) {}
    template <typename A, typename B>
    tvec2(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
    template <typename U, precision Q>
    explicit tvec2(tvec2<U, Q> const& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)) {}

    tvec2 operator+(tvec2 const& o) const { return tvec2(x + o.x, y + o.y); }
    tvec2 operator-(tvec2 const& o) const { return tvec2(x - o.x, y - o.y); }
    tvec2 operator*(tvec2 const& o) const { return tvec2(x * o.x, y * o.y); }
    tvec2 operator/(tvec2 const& o) const { return tvec2(x / o.x, y / o.y); }
    tvec2 operator-() const { return tvec2(-x, -y); }
    bool operator==(tvec2 const& o) const { return x == o.x && y == o.y; }
    bool operator!=(tvec2 const& o) const { return !(*this == o); }
};

typedef tvec2<bool>          bvec2;
typedef tvec2<float>         vec2;
typedef tvec2<std::int32_t>  i32vec2;
typedef tvec2<std::uint32_t> u32vec2;
typedef tvec2<std::uint32_t> uvec2;
typedef tvec2<std::uint8_t>  u8vec2;

template <typename T, precision P>
inline bvec2 lessThan(tvec2<T, P> const& a, tvec2<T, P> const& b) { return bvec2(a.x < b.x, a.y < b.y); }
template <typename T, precision P>
inline bvec2 lessThanEqual(tvec2<T, P> const& a, tvec2<T, P> const& b) { return bvec2(a.x <= b.x, a.y <= b.y); }
inline bool all(bvec2 const& v) { return v.x && v.y; }

// Scalar helpers reached through `using namespace glm;` in eikonal.h.
template <typename T> inline T min(T a, T b) { return std::min(a, b); }
template <typename T> inline T max(T a, T b) { return std::max(a, b); }
template <typename T> inline T sqrt(T v) { return std::sqrt(v); }
template <typename T> inline bool isinf(T v) { return std::isinf(v); }

}  // namespace glm

using glm::u8;
using glm::u32;

template <typename T>
using optional = std::optional<T>;

namespace cl {
struct Device {};
struct Context {};
struct CommandQueue {};
struct Program {};
}  // namespace cl

template <typename T, size_t K>
size_t length_of(T (&)[K]) { return K; }
