// Compatibility header for Geometry.h of the reference (Geometry.h:1-32, Geometry.cpp:22-42).
#ifndef GEOMETRY_H
#define GEOMETRY_H

#include <math.h>

struct Point_3
{
    float x, y, z;

    Point_3(float x_i, float y_i, float z_i) : x(x_i), y(y_i), z(z_i) {}

    bool operator==(const Point_3& a) const { return a.x == x && a.y == y && a.z == z; }

    // v / |v| in float
    void normaliseVector()
    {
        const float norm = sqrtf((x * x) + (y * y) + (z * z));
        x /= norm;
        y /= norm;
        z /= norm;
    }
};

// quaternion rotation of `vector` about `axis` by `angle` radians
Point_3 rotateVectorAroundAxis(Point_3 axis, Point_3 vector, float angle);

#endif
