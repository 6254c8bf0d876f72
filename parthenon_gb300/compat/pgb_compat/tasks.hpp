// Package-facing compatibility layer: task lists.
//
// Reference: src/tasks/tasks.hpp:158-527 (TaskID, TaskList::AddTask(dep, fn, args...),
// TaskRegion, TaskCollection), src/tasks/tasks.cpp:45-153 (execution: tasks run when
// their dependencies are complete; `incomplete` tasks are polled again; `fail` stops the
// collection; regions run in order), src/basic_types.hpp (TaskListStatus).
//
// Tasks run on the host thread in dependency order; the work they enqueue is
// stream-ordered on the layer's CUDA stream, so a task's kernels follow its
// dependencies' kernels without host synchronisation.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <type_traits>
#include <memory>
#include <set>
#include <tuple>
#include <utility>
#include <vector>

#include "core.hpp"

// task labels: the function's spelling, then the function (src/tasks/tasks.hpp:39)
#ifndef TF
#define TF(...) std::string(#__VA_ARGS__), __VA_ARGS__
#endif

namespace parthenon {

enum class TaskListStatus { complete, fail, running, nothing_to_do };

// A set of task ids; TaskID(0) (or a default TaskID) depends on nothing.
class TaskID {
 public:
  TaskID() = default;
  explicit TaskID(int id) {
    if (id > 0) ids_.insert(id);
  }
  TaskID operator|(const TaskID &o) const {
    TaskID r(*this);
    r.ids_.insert(o.ids_.begin(), o.ids_.end());
    return r;
  }
  TaskID &operator|=(const TaskID &o) {
    ids_.insert(o.ids_.begin(), o.ids_.end());
    return *this;
  }
  bool operator==(const TaskID &o) const { return ids_ == o.ids_; }
  const std::set<int> &ids() const { return ids_; }
  const std::set<int> &GetIDs() const { return ids_; }  // tasks.hpp TaskID::GetIDs
  bool empty() const { return ids_.empty(); }

 private:
  std::set<int> ids_;
};

// src/tasks/tasks.hpp:52-80: how a task takes part in its region. One partition per
// region runs here, so local and global synchronisation are the dependency order
// itself; `completion` tasks decide whether an iterating sublist goes round again.
class TaskQualifier {
 public:
  using qualifier_t = uint64_t;
  TaskQualifier() = delete;
  TaskQualifier(const qualifier_t n) : flags(n) {}  // NOLINT(runtime/explicit)
  static inline constexpr qualifier_t normal{0};
  static inline constexpr qualifier_t local_sync{1 << 0};
  static inline constexpr qualifier_t global_sync{1 << 1};
  static inline constexpr qualifier_t completion{1 << 2};
  static inline constexpr qualifier_t once_per_region{1 << 3};
  bool LocalSync() const { return flags & local_sync; }
  bool GlobalSync() const { return flags & global_sync; }
  bool Completion() const { return flags & completion; }
  bool Once() const { return flags & once_per_region; }

 private:
  qualifier_t flags;
};

template <class T>
struct compat_is_tuple : std::false_type {};
template <class... Ts>
struct compat_is_tuple<std::tuple<Ts...>> : std::true_type {};

class TaskList {
 public:
  TaskList() = default;
  TaskList(int min_iters, int max_iters) : min_iters_(min_iters), max_iters_(max_iters) {}

  // AddTask([qualifier,] dep, [label | (label, verbosity, fn) tuple,] fn, args...): fn
  // (a callable or a member-function pointer followed by its object) must return a
  // TaskStatus; the arguments are stored by value
  template <class Arg1, class... Args>
  TaskID AddTask(const TaskID &dep, Arg1 &&a1, Args &&...args) {
    return AddTask(TaskQualifier::normal, dep, std::forward<Arg1>(a1), std::forward<Args>(args)...);
  }
  template <class Arg1, class... Args>
  TaskID AddTask(const TaskQualifier tq, const TaskID &dep, Arg1 &&a1, Args &&...args) {
    if constexpr (std::is_invocable<Arg1, Args...>::value) {
      return add(tq, dep, std::forward<Arg1>(a1), std::forward<Args>(args)...);
    } else if constexpr (std::is_convertible<Arg1, std::string>::value) {
      return add(tq, dep, std::forward<Args>(args)...);  // a label
    } else if constexpr (compat_is_tuple<std::decay_t<Arg1>>::value) {
      return add(tq, dep, std::get<2>(a1), std::forward<Args>(args)...);
    } else {
      static_assert(std::is_invocable<Arg1, Args...>::value, "AddTask: bad signature");
      return TaskID();
    }
  }
  // A list that runs after `dep` and, when its tasks are done, runs again while a
  // completion task asked to iterate (at least min, at most max times); the returned id
  // completes with it (src/tasks/tasks.hpp:342-347)
  std::pair<TaskList &, TaskID> AddSublist(const TaskID &dep, std::pair<int, int> minmax_iters) {
    sublists_.push_back(std::make_unique<TaskList>(minmax_iters.first, minmax_iters.second));
    TaskList *sub = sublists_.back().get();
    const TaskID id = add(TaskQualifier::normal, dep, [sub]() { return sub->RunIterations(); });
    return {*sub, id};
  }
  // one pass over the tasks whose dependencies are done; returns the list's status
  TaskListStatus Step() {
    if (failed_) return TaskListStatus::fail;
    bool ran = true;
    while (ran) {
      ran = false;
      for (auto &t : tasks_) {
        if (t.done || !ready(t)) continue;
        const TaskStatus st = t.fn();
        if (st == TaskStatus::fail) {
          failed_ = true;
          return TaskListStatus::fail;
        }
        if (st == TaskStatus::complete || st == TaskStatus::iterate) {
          t.done = true;
          t.status = st;
          ran = true;
        }
      }
    }
    for (auto &t : tasks_)
      if (!t.done) return TaskListStatus::running;
    return TaskListStatus::complete;
  }
  // the whole list, iterated as a sublist: complete, fail, or incomplete while a task
  // waits
  TaskStatus RunIterations() {
    while (true) {
      const TaskListStatus st = Step();
      if (st == TaskListStatus::fail) return TaskStatus::fail;
      if (st != TaskListStatus::complete) return TaskStatus::incomplete;
      ++iter_;
      bool again = false;
      for (auto &t : tasks_)
        if (t.completion && t.status == TaskStatus::iterate) again = true;
      if (iter_ < min_iters_) again = true;
      if (!again || iter_ >= max_iters_) return TaskStatus::complete;
      for (auto &t : tasks_) t.done = false;
    }
  }
  bool Empty() const { return tasks_.empty(); }

 private:
  struct Task {
    int id;
    TaskID dep;
    std::function<TaskStatus()> fn;
    bool done;
    bool completion;
    TaskStatus status;
  };
  template <class F, class... Args>
  TaskID add(const TaskQualifier tq, const TaskID &dep, F &&fn, Args &&...args) {
    auto call = [f = std::forward<F>(fn), tup = std::make_tuple(std::forward<Args>(args)...)]() mutable {
      return std::apply([&f](auto &...a) { return static_cast<TaskStatus>(std::invoke(f, a...)); }, tup);
    };
    tasks_.push_back(Task{(int)tasks_.size() + 1, dep, std::function<TaskStatus()>(std::move(call)), false,
                          tq.Completion(), TaskStatus::incomplete});
    return TaskID(tasks_.back().id);
  }
  bool ready(const Task &t) const {
    for (int d : t.dep.ids())
      if (d < 1 || d > (int)tasks_.size() || !tasks_[d - 1].done) return false;
    return true;
  }
  std::vector<Task> tasks_;
  std::vector<std::unique_ptr<TaskList>> sublists_;
  bool failed_ = false;
  int min_iters_ = 1, max_iters_ = 1, iter_ = 0;
};

class TaskRegion {
 public:
  explicit TaskRegion(int n) : lists_(n) {}
  TaskList &operator[](int i) { return lists_.at(i); }
  int size() const { return (int)lists_.size(); }
  // lists advance in turn until all are complete (a list waiting on an `incomplete`
  // task does not block the others); gives up after max_passes without progress
  TaskListStatus Execute(int max_passes = 1000000) {
    for (int pass = 0; pass < max_passes; ++pass) {
      bool all = true;
      for (auto &l : lists_) {
        const TaskListStatus st = l.Step();
        if (st == TaskListStatus::fail) return st;
        if (st != TaskListStatus::complete) all = false;
      }
      if (all) return TaskListStatus::complete;
    }
    return TaskListStatus::fail;
  }

 private:
  std::vector<TaskList> lists_;
};

class TaskCollection {
 public:
  TaskRegion &AddRegion(int n) {
    regions_.push_back(std::make_unique<TaskRegion>(n));
    return *regions_.back();
  }
  TaskListStatus Execute() {
    for (auto &r : regions_) {
      const TaskListStatus st = r->Execute();
      if (st == TaskListStatus::fail) return st;
    }
    return TaskListStatus::complete;
  }

 private:
  std::vector<std::unique_ptr<TaskRegion>> regions_;
};

}  // namespace parthenon
