// Writes key sequences on which std::sort (libstdc++'s introsort) runs out of
// its depth budget and finishes segments with its heap sort: the inputs of
// tests/test_gpu_scene_prep.py::test_reference_bvh_heap_sort, which checks
// that the device build of the reference BVH takes the same path.
//
// The sequences come from McIlroy's adversary ("A killer adversary for
// quicksort", Software: Practice and Experience 29(4), 1999): std::sort runs
// on n items whose values are undecided ("gas") until a comparison needs
// them; of two gas items compared, the one the comparator has seen as the
// pivot candidate is frozen to the next smallest value.  The answers are
// consistent with the final values, so sorting those values replays the
// same comparisons.
//
//   g++ -O2 -std=c++17 -o /tmp/killer tests/golden/make_introsort_killer.cpp
//   /tmp/killer 1000 > tests/golden/introsort_killer_1000.txt
//   /tmp/killer 3000 > tests/golden/introsort_killer_3000.txt
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <vector>

int main(int argc, char** argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 1000;
  const int gas = n;  // larger than every frozen value
  std::vector<int> val(static_cast<size_t>(n), gas), idx(static_cast<size_t>(n));
  std::iota(idx.begin(), idx.end(), 0);
  int nsolid = 0, candidate = 0;
  auto freeze = [&](int i) { val[size_t(i)] = nsolid++; };
  auto less = [&](int x, int y) {
    if (val[size_t(x)] == gas && val[size_t(y)] == gas) {
      if (x == candidate) freeze(x);
      else freeze(y);
    }
    if (val[size_t(x)] == gas) candidate = x;
    else if (val[size_t(y)] == gas) candidate = y;
    return val[size_t(x)] < val[size_t(y)];
  };
  std::sort(idx.begin(), idx.end(), less);
  for (int i = 0; i < n; ++i)
    if (val[size_t(i)] == gas) freeze(i);
  for (int i = 0; i < n; ++i) std::printf("%d\n", val[size_t(i)]);
  return 0;
}
