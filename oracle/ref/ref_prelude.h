/*
 * Forced-include prelude for the headless build of the reference solver
 * (ByungJoonLee/2D_Engine) that the oracle tests use as ground truth.
 *
 * The reference was written for MSVC, which does not look inside uninstantiated
 * template members.  GCC does, and stops at a handful of typos in members that
 * the hot path never calls.  Instead of editing the read-only sources, this
 * prelude gives those names something to bind to:
 *   - ARRAY.h:105 `values_input`, VECTOR_ND.h:233 `max_abs`,
 *     FIELD_STRUCTURE_2D.h:351 `value`, DYNAMIC_ARRAY.h:86,115,116,148
 *     `num_elements`/`valuess`/`num_of_elemetns`: file-scope dummies.  Any real
 *     parameter or member of the same name shadows them, so no live code changes.
 *   - ARRAY_2D.h:75-77 names a parameter `Initialize` and then calls the member
 *     `Initialize(...)`: the function-like macro below renames every *call and
 *     declaration* `Initialize(` to `Initialize_(` uniformly, which leaves the
 *     parameter (not followed by '(') alone.
 *   - ARRAY_1D.h:110 returns CLAMP(int...) as a VI: CLAMP is redefined to yield
 *     the same value as MACROS.h:14 through a wrapper that also converts to VI.
 * None of this touches an arithmetic expression of the hot path.
 */
#pragma once
#include <cstring>
#include <type_traits>

#include "MACROS.h"

#undef CLAMP
template <class R>
struct ref_clamp_result {
  R v;
  operator R() const { return v; }
  template <class U, class = typename std::enable_if<!std::is_arithmetic<U>::value>::type>
  operator U() const { return U(v, v); }
};
template <class A, class B, class C>
inline ref_clamp_result<typename std::common_type<A, B, C>::type> ref_clamp(const A& a, const B& b, const C& c) {
  typedef typename std::common_type<A, B, C>::type R;
  return ref_clamp_result<R>{a < b ? (R)b : (a > c ? (R)c : (R)a)};
}
#define CLAMP(v, lo, hi) (ref_clamp((v), (lo), (hi)))

static double values_input;
static double max_abs;
static double* value;
static int num_elements;
static int num_of_elemetns;
static int* valuess;

#define Initialize(...) Initialize_(__VA_ARGS__)
