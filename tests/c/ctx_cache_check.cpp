// CPU check of the per-context address cache used by the allocation-free
// adjoint (ddc-svd_gb300/csrc/ctx_cache.hpp): values are kept per context
// id, a miss calls the maker once, a failing maker caches nothing, and a
// full table evicts its oldest entry without ever answering with another
// context's value.  Compiled and run by tests/test_c_abi.py; prints "ok".
#include <stdio.h>

#include "ctx_cache.hpp"

static int calls = 0;

#define CHECK(c)                                          \
  do {                                                    \
    if (!(c)) {                                           \
      printf("FAIL line %d: %s\n", __LINE__, #c);          \
      return 1;                                           \
    }                                                     \
  } while (0)

int main() {
  ddcsvd::CtxValueCache<4> cache;
  static char objs[16];
  auto maker = [](unsigned long long id) {
    return [id](void** v) {
      calls++;
      *v = &objs[id % 16];
      return 0;
    };
  };
  void* p = nullptr;
  CHECK(cache.get(7, &p, maker(7)) == 0 && p == &objs[7] && calls == 1);
  CHECK(cache.get(7, &p, maker(7)) == 0 && p == &objs[7] && calls == 1);  // hit: no second lookup
  CHECK(cache.get(8, &p, maker(8)) == 0 && p == &objs[8] && calls == 2);  // another context: its own value
  // a failing maker passes its status through and caches nothing
  CHECK(cache.get(9, &p, [](void**) { return 2; }) == 2);
  CHECK(cache.size() == 2);
  CHECK(cache.get(9, &p, maker(9)) == 0 && p == &objs[9] && calls == 3);
  // fill past capacity: 7 (oldest) makes room, everyone else still answers with its own value
  CHECK(cache.get(10, &p, maker(10)) == 0 && cache.size() == 4);
  CHECK(cache.get(11, &p, maker(11)) == 0 && p == &objs[11] && cache.size() == 4);
  const int before = calls;
  CHECK(cache.get(8, &p, maker(8)) == 0 && p == &objs[8] && calls == before);
  CHECK(cache.get(7, &p, maker(7)) == 0 && p == &objs[7] && calls == before + 1);  // evicted: looked up again
  // a context id that equals an old handle value but is new gets a fresh lookup
  CHECK(cache.get(12, &p, maker(12)) == 0 && p == &objs[12] && calls == before + 2);
  printf("ok\n");
  return 0;
}
