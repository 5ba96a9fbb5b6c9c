// lowlevel.h -- single-threaded stand-in for the low-level runtime API that
// LegionOrigins' benchmarks/reductions/reducetest.cc was written against
// (namespace RegionRuntime::LowLevel; the runtime shipped beside it has moved
// on to LegionRuntime::LowLevel and no longer matches).  Test infrastructure
// only: it lets the benchmark's own source compile and run unmodified so its
// histograms can be dumped as golden vectors.  Nothing in the product links
// it.
//
// Semantics kept from the shared-memory runtime (runtime/shared_lowlevel.cc):
//   - a normal instance holds LHS values; reduce<REDOP> applies in place;
//   - a fold instance holds RHS values initialised to REDOP::identity and
//     folds into them; copy_to a normal instance applies every element
//     (shared_lowlevel.cc:2706-2712);
//   - a list instance appends (ptr, rhs) entries up to its capacity; copy_to
//     a normal instance applies the entries in order and leaves the list as
//     it is (apply_list, shared_lowlevel.cc:2744-2762);
//   - normal-to-normal copy_to copies every element.
// Tasks run synchronously inside spawn() on one processor; events and locks
// are therefore trivially satisfied.  Log output is discarded, as with the
// benchmark's OUTPUT_LEVEL=LEVEL_NONE build.
//
// When CKT_REFSHIM_DUMP names a file, Machine::run writes the contents of the
// first normal instance the program created (the benchmark's master
// histogram) to it as raw bytes after the top-level task returns.
#ifndef CKT_REFSHIM_LOWLEVEL_H
#define CKT_REFSHIM_LOWLEVEL_H

#include <sys/time.h>

#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <vector>

namespace RegionRuntime {

class Logger {
 public:
  class Category {
   public:
    explicit Category(const char *) {}
    void info(const char *, ...) const {}
    void debug(const char *, ...) const {}
    void warning(const char *, ...) const {}
    void error(const char *, ...) const {}
  };
};

namespace LowLevel {

typedef unsigned ReductionOpID;

class Event {
 public:
  unsigned id = 0;
  static const Event NO_EVENT;
  bool operator<(const Event &o) const { return id < o.id; }
  bool operator==(const Event &o) const { return id == o.id; }
  void wait() const {}
  static Event merge_events(const std::set<Event> &) { return Event(); }
};
inline const Event Event::NO_EVENT = Event();

class UserEvent : public Event {
 public:
  static UserEvent create_user_event() { return UserEvent(); }
  void trigger() const {}
};

class Lock {
 public:
  unsigned id = 0;
  static Lock create_lock() { return Lock(); }
  Event lock() const { return Event(); }
  void unlock(Event = Event::NO_EVENT) const {}
};

class Memory {
 public:
  unsigned id = 1;
  bool operator<(const Memory &o) const { return id < o.id; }
};

class Processor;
typedef void (*TaskFuncPtr)(const void *args, size_t arglen, Processor proc);

class Processor {
 public:
  unsigned id = 1;
  enum { TASK_ID_PROCESSOR_INIT = 1, TASK_ID_PROCESSOR_SHUTDOWN = 2, TASK_ID_FIRST_AVAILABLE = 4 };
  typedef std::map<unsigned, TaskFuncPtr> TaskIDTable;
  bool operator<(const Processor &o) const { return id < o.id; }
  Event spawn(unsigned func_id, const void *args, size_t arglen,
              Event wait_on = Event::NO_EVENT) const;
};

template <class T>
struct ptr_t {
  unsigned value;
  ptr_t(unsigned v = 0) : value(v) {}
};

// Type-erased reduction operator: what copy_to needs to apply a fold or a
// list instance without knowing REDOP.
class ReductionOpUntyped {
 public:
  size_t sizeof_lhs = 0, sizeof_rhs = 0;
  void (*apply)(void *lhs, const void *rhs) = nullptr;
  void (*init)(void *rhs) = nullptr;
  template <class REDOP>
  static ReductionOpUntyped *create_reduction_op();
};
typedef std::map<ReductionOpID, const ReductionOpUntyped *> ReductionOpTable;

namespace shim {
template <class REDOP>
struct RedopFns {
  typedef typename REDOP::LHS L;
  typedef typename REDOP::RHS R;
  static void apply(void *l, const void *r) {
    R v;
    std::memcpy(&v, r, sizeof(R));
    REDOP::template apply<true>(*static_cast<L *>(l), v);
  }
  static void init(void *r) {
    const R id = REDOP::identity;
    std::memcpy(r, &id, sizeof(R));
  }
};

enum Kind { NORMAL, FOLD, LIST };

struct Instance {
  Kind kind = NORMAL;
  size_t elems = 0, elem_size = 0;
  std::vector<unsigned char> data;  // NORMAL: LHS[elems]; FOLD: RHS[elems]
  const ReductionOpUntyped *op = nullptr;
  size_t capacity = 0;                      // LIST
  std::vector<unsigned> list_ptr;           // LIST entries: pointer
  std::vector<unsigned char> list_rhs;      // LIST entries: RHS bytes
};

inline ReductionOpTable &redops() {
  static ReductionOpTable t;
  return t;
}
inline Instance *&first_normal() {
  static Instance *p = nullptr;
  return p;
}
[[noreturn]] inline void die(const char *msg) {
  std::fprintf(stderr, "refshim: %s\n", msg);
  std::exit(2);
}
}  // namespace shim

template <class REDOP>
ReductionOpUntyped *ReductionOpUntyped::create_reduction_op() {
  ReductionOpUntyped *op = new ReductionOpUntyped;
  op->sizeof_lhs = sizeof(typename REDOP::LHS);
  op->sizeof_rhs = sizeof(typename REDOP::RHS);
  op->apply = &shim::RedopFns<REDOP>::apply;
  op->init = &shim::RedopFns<REDOP>::init;
  return op;
}

struct AccessorGeneric {};
struct AccessorArray {};
struct AccessorArrayReductionFold {};
struct AccessorReductionList {};

template <class T, class AT = AccessorGeneric>
class RegionInstanceAccessor {
 public:
  shim::Instance *impl = nullptr;

  template <class AT2>
  RegionInstanceAccessor<T, AT2> convert() const {
    RegionInstanceAccessor<T, AT2> r;
    r.impl = impl;
    return r;
  }
  T read(ptr_t<T> p) const {
    if (impl->kind != shim::NORMAL) shim::die("read from a reduction instance");
    T v;
    std::memcpy(&v, impl->data.data() + (size_t)p.value * sizeof(T), sizeof(T));
    return v;
  }
  void write(ptr_t<T> p, const T &v) const {
    if (impl->kind != shim::NORMAL) shim::die("write to a reduction instance");
    std::memcpy(impl->data.data() + (size_t)p.value * sizeof(T), &v, sizeof(T));
  }
  template <class REDOP>
  void reduce(ptr_t<T> p, typename REDOP::RHS rhs) const {
    typedef typename REDOP::LHS L;
    typedef typename REDOP::RHS R;
    if (p.value >= impl->elems) shim::die("reduction pointer out of range");
    switch (impl->kind) {
      case shim::NORMAL:
        REDOP::template apply<true>(reinterpret_cast<L *>(impl->data.data())[p.value], rhs);
        break;
      case shim::FOLD:
        REDOP::template fold<true>(reinterpret_cast<R *>(impl->data.data())[p.value], rhs);
        break;
      case shim::LIST: {
        if (impl->list_ptr.size() >= impl->capacity) shim::die("reduction list overflow");
        impl->list_ptr.push_back(p.value);
        const unsigned char *b = reinterpret_cast<const unsigned char *>(&rhs);
        impl->list_rhs.insert(impl->list_rhs.end(), b, b + sizeof(R));
        break;
      }
    }
  }
};

template <class T>
class RegionInstance {
 public:
  shim::Instance *impl = nullptr;

  RegionInstanceAccessor<T, AccessorGeneric> get_accessor() const {
    RegionInstanceAccessor<T, AccessorGeneric> a;
    a.impl = impl;
    return a;
  }
  Event copy_to(RegionInstance<T> dst) const {
    shim::Instance *s = impl, *d = dst.impl;
    if (d->kind != shim::NORMAL) shim::die("copy into a reduction instance is not modelled");
    switch (s->kind) {
      case shim::NORMAL:
        std::memcpy(d->data.data(), s->data.data(), d->data.size());
        break;
      case shim::FOLD:
        for (size_t i = 0; i < s->elems; i++)
          s->op->apply(d->data.data() + i * s->op->sizeof_lhs,
                       s->data.data() + i * s->op->sizeof_rhs);
        break;
      case shim::LIST:
        for (size_t i = 0; i < s->list_ptr.size(); i++)
          s->op->apply(d->data.data() + (size_t)s->list_ptr[i] * s->op->sizeof_lhs,
                       s->list_rhs.data() + i * s->op->sizeof_rhs);
        break;
    }
    return Event();
  }
};

template <class T>
class RegionMetaData {
 public:
  size_t elems = 0;

  static RegionMetaData<T> create_region(size_t n) {
    RegionMetaData<T> r;
    r.elems = n;
    return r;
  }
  RegionInstance<T> create_instance(Memory) const {
    shim::Instance *i = new shim::Instance;
    i->kind = shim::NORMAL;
    i->elems = elems;
    i->elem_size = sizeof(T);
    i->data.assign(elems * sizeof(T), 0);
    if (!shim::first_normal()) shim::first_normal() = i;
    RegionInstance<T> r;
    r.impl = i;
    return r;
  }
  RegionInstance<T> create_instance(Memory, ReductionOpID redop) const {
    const ReductionOpUntyped *op = lookup(redop);
    shim::Instance *i = new shim::Instance;
    i->kind = shim::FOLD;
    i->elems = elems;
    i->elem_size = op->sizeof_rhs;
    i->op = op;
    i->data.resize(elems * op->sizeof_rhs);
    for (size_t k = 0; k < elems; k++) op->init(i->data.data() + k * op->sizeof_rhs);
    RegionInstance<T> r;
    r.impl = i;
    return r;
  }
  RegionInstance<T> create_instance(Memory, ReductionOpID redop, off_t list_size,
                                    RegionInstance<T>) const {
    shim::Instance *i = new shim::Instance;
    i->kind = shim::LIST;
    i->elems = elems;
    i->op = lookup(redop);
    i->capacity = (size_t)list_size;
    RegionInstance<T> r;
    r.impl = i;
    return r;
  }
  void destroy_instance(RegionInstance<T> inst) const {
    if (inst.impl == shim::first_normal()) shim::die("the dumped instance was destroyed");
    delete inst.impl;
  }

 private:
  static const ReductionOpUntyped *lookup(ReductionOpID id) {
    auto it = shim::redops().find(id);
    if (it == shim::redops().end()) shim::die("unknown reduction operator");
    return it->second;
  }
};

class Machine {
 public:
  struct ProcessorMemoryAffinity {
    Processor p;
    Memory m;
    unsigned bandwidth;
    unsigned latency;
  };
  enum RunStyle { ONE_TASK_ONLY, ONE_TASK_PER_NODE, ONE_TASK_PER_PROC };

  Machine(int *, char ***, const Processor::TaskIDTable &tasks, const ReductionOpTable &redops,
          bool) : tasks_(tasks) {
    shim::redops() = redops;
    procs_.insert(Processor());
    instance() = this;
  }
  static Machine *get_machine() { return instance(); }
  const std::set<Processor> &get_all_processors() const { return procs_; }
  int get_proc_mem_affinity(std::vector<ProcessorMemoryAffinity> &result,
                            Processor = Processor()) const {
    ProcessorMemoryAffinity a;
    a.p = Processor();
    a.m = Memory();
    a.bandwidth = 1;
    a.latency = 1;
    result.push_back(a);
    return 1;
  }
  void run(unsigned task_id, RunStyle = ONE_TASK_ONLY, const void *args = nullptr,
           size_t arglen = 0) {
    Processor().spawn(task_id, args, arglen);
    if (const char *path = std::getenv("CKT_REFSHIM_DUMP")) {
      shim::Instance *m = shim::first_normal();
      if (!m) shim::die("no instance to dump");
      FILE *f = std::fopen(path, "wb");
      if (!f || std::fwrite(m->data.data(), 1, m->data.size(), f) != m->data.size())
        shim::die("dump failed");
      std::fclose(f);
    }
    std::exit(0);
  }
  TaskFuncPtr task(unsigned id) const {
    auto it = tasks_.find(id);
    return it == tasks_.end() ? nullptr : it->second;
  }

 private:
  static Machine *&instance() {
    static Machine *m = nullptr;
    return m;
  }
  Processor::TaskIDTable tasks_;
  std::set<Processor> procs_;
};

inline Event Processor::spawn(unsigned func_id, const void *args, size_t arglen, Event) const {
  if (func_id == 0) return Event();  // the shutdown "kill pill"
  TaskFuncPtr f = Machine::get_machine()->task(func_id);
  if (!f) shim::die("spawn of an unregistered task");
  f(args, arglen, *this);
  return Event();
}

class Clock {
 public:
  static double abs_time() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
  }
};

}  // namespace LowLevel
}  // namespace RegionRuntime

#endif
