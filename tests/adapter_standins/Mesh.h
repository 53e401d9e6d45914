// Stand-in for the reference's src/Mesh.h: vertex positions and faces.
#ifndef MESH_H
#define MESH_H

#include <Eigen/Core>

struct Mesh {
  Eigen::VectorXd vertices;
  Eigen::Matrix3Xi faces;
};

#endif
