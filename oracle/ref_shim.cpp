// C entry points over the reference's own sources compiled by
// oracle/build_ref.py into oracle/_ref/libhg_ref.so (test infrastructure
// only): the oracle's restatements are checked against these.
#include "CircleRectangleIntersection.h"

extern "C" double hgr_circle_rectangle_area(double x0, double x1, double y0, double y1,
                                            double cx, double cy, double r) {
  return circleRectangleIntersectionArea(x0, x1, y0, y1, cx, cy, r);
}
