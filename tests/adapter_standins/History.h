// Stand-in for the reference's src/History.h: per-vertex position histories.
// Only the two-entry form (start at time 0, end at time 1) is built here.
#ifndef HISTORY_H
#define HISTORY_H

#include <Eigen/Core>
#include <vector>

struct HistoryEntry {
  double time;
  Eigen::Vector3d pos;
};

class History {
 public:
  explicit History(const Eigen::VectorXd &qstart) : history_(qstart.size() / 3) {
    for (size_t v = 0; v < history_.size(); v++) {
      HistoryEntry e;
      e.time = 0.0;
      e.pos = Eigen::Vector3d(qstart[3 * v], qstart[3 * v + 1], qstart[3 * v + 2]);
      history_[v].push_back(e);
    }
  }
  void finishHistory(const Eigen::VectorXd &qend) {
    for (size_t v = 0; v < history_.size(); v++) {
      HistoryEntry e;
      e.time = 1.0;
      e.pos = Eigen::Vector3d(qend[3 * v], qend[3 * v + 1], qend[3 * v + 2]);
      history_[v].push_back(e);
    }
  }
  const std::vector<HistoryEntry> &getVertexHistory(int vert) const { return history_[vert]; }

 private:
  std::vector<std::vector<HistoryEntry> > history_;
};

#endif
