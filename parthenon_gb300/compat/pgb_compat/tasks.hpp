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

#include <functional>
#include <memory>
#include <set>
#include <tuple>
#include <utility>
#include <vector>

#include "core.hpp"

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
  bool empty() const { return ids_.empty(); }

 private:
  std::set<int> ids_;
};

class TaskList {
 public:
  // fn(args...) must return a TaskStatus; the arguments are stored by value
  template <class F, class... Args>
  TaskID AddTask(const TaskID &dep, F &&fn, Args &&...args) {
    auto call = [f = std::forward<F>(fn), tup = std::make_tuple(std::forward<Args>(args)...)]() mutable {
      return std::apply([&f](auto &...a) { return static_cast<TaskStatus>(f(a...)); }, tup);
    };
    tasks_.push_back(Task{(int)tasks_.size() + 1, dep, std::function<TaskStatus()>(std::move(call)), false});
    return TaskID(tasks_.back().id);
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
          ran = true;
        }
      }
    }
    for (auto &t : tasks_)
      if (!t.done) return TaskListStatus::running;
    return TaskListStatus::complete;
  }
  bool Empty() const { return tasks_.empty(); }

 private:
  struct Task {
    int id;
    TaskID dep;
    std::function<TaskStatus()> fn;
    bool done;
  };
  bool ready(const Task &t) const {
    for (int d : t.dep.ids())
      if (d < 1 || d > (int)tasks_.size() || !tasks_[d - 1].done) return false;
    return true;
  }
  std::vector<Task> tasks_;
  bool failed_ = false;
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
