// Compatibility header for Model.h of the reference (Model.h, Model.cpp:22-91) on the library's
// mesh front end (lbm_mesh_*).  The reference's CGAL point type in isPointInsideModel and
// reflectionVector is Point_3 here; CGAL is not used.
#pragma once

#include <string>

#include "Geometry.h"

struct lbm_mesh;

// the parts of the reference's Surface_mesh and Iso_cuboid_3 that callers use
struct MeshData
{
    long long vertices = 0, faces = 0;
    long long number_of_vertices() const { return vertices; }
    long long number_of_faces() const { return faces; }
};

struct BoundingBox
{
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    float xmin() const { return lo[0]; }
    float ymin() const { return lo[1]; }
    float zmin() const { return lo[2]; }
    float xmax() const { return hi[0]; }
    float ymax() const { return hi[1]; }
    float zmax() const { return hi[2]; }
};

class Model
{
public:
    Model() = default;
    ~Model();
    Model(const Model&) = delete;
    Model& operator=(const Model&) = delete;

    // Wavefront OBJ; a missing file leaves the model empty (as the reference)
    void importModel(std::string filename);

    bool isModelClosed();

    // inside or on the surface; false for an invalid model
    bool isPointInsideModel(Point_3 point);

    const MeshData& getMesh() const { return modelMesh; }

    // true when the model is not a closed triangle mesh
    bool checkError() { return !meshValid; }

    BoundingBox bounding_box();

    Point_3 reflectionVector(Point_3 point_1, Point_3 point_2);

    // the library's mesh handle (nullptr before a successful import)
    lbm_mesh* handle() const { return mesh; }

private:
    lbm_mesh* mesh = nullptr;
    MeshData modelMesh;
    bool meshValid = true;
};
