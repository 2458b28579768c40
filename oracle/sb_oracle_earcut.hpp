// Ear-clipping triangulator restated for the CPU oracle (test infrastructure only).
//
// Follows the steps of the modified mapbox earcut vendored by the reference
// (thirdparty/earcut.hpp/include/mapbox/earcut.hpp): linked ring construction with winding normalisation
// (:210-245), point filtering (:248-271), the three-pass ear loop (:274-326), plain and z-order ear tests
// (:329-388), local self-intersection cure (:391-415), split fallback (:418-442), hole elimination with
// Eberly's bridge search (:445-544), z-order curve indexing and Tatham's list merge sort (:552-658), and
// the reference author's change to area(): values within DBL_EPSILON of zero count as zero (:694-699).
// Nodes live in a vector and are linked by index instead of by pointer.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

namespace port {

class Earcut {
public:
    std::vector<int64_t> indices;

    void run(const std::vector<std::vector<std::array<double, 2>>> &rings)
    {
        indices.clear();
        nodes.clear();
        vertices = 0;
        if (rings.empty())
            return;
        int threshold = 80;
        for (size_t r = 0; threshold >= 0 && r < rings.size(); ++r)
            threshold -= (int)rings[r].size();
        int outer = linkedList(rings[0], true);
        if (outer < 0 || N(outer).prev == N(outer).next)
            return;
        if (rings.size() > 1)
            outer = eliminateHoles(rings, outer);
        hashing = threshold < 0;
        if (hashing) {
            int p = N(outer).next;
            minX = maxX = N(outer).x;
            minY = maxY = N(outer).y;
            do {
                double x = N(p).x, y = N(p).y;
                minX = std::min(minX, x);
                minY = std::min(minY, y);
                maxX = std::max(maxX, x);
                maxY = std::max(maxY, y);
                p = N(p).next;
            } while (p != outer);
            invSize = std::max(maxX - minX, maxY - minY);
            invSize = invSize != 0.0 ? (1.0 / invSize) : 0.0;
        }
        earcutLinked(outer, 0);
    }

private:
    struct Node {
        int64_t i;
        double x, y;
        int prev = -1, next = -1;
        int32_t z = 0;
        int prevZ = -1, nextZ = -1;
        bool steiner = false;
    };
    std::vector<Node> nodes;
    int64_t vertices = 0;
    bool hashing = false;
    double minX = 0, maxX = 0, minY = 0, maxY = 0, invSize = 0;

    Node &N(int k) { return nodes[(size_t)k]; }

    int newNode(int64_t i, double x, double y)
    {
        Node n;
        n.i = i;
        n.x = x;
        n.y = y;
        nodes.push_back(n);
        return (int)nodes.size() - 1;
    }

    int insertNode(int64_t i, double x, double y, int last)
    {
        int p = newNode(i, x, y);
        if (last < 0) {
            N(p).prev = p;
            N(p).next = p;
        } else {
            N(p).next = N(last).next;
            N(p).prev = last;
            N(N(last).next).prev = p;
            N(last).next = p;
        }
        return p;
    }

    void removeNode(int p)
    {
        N(N(p).next).prev = N(p).prev;
        N(N(p).prev).next = N(p).next;
        if (N(p).prevZ >= 0)
            N(N(p).prevZ).nextZ = N(p).nextZ;
        if (N(p).nextZ >= 0)
            N(N(p).nextZ).prevZ = N(p).prevZ;
    }

    int linkedList(const std::vector<std::array<double, 2>> &pts, bool clockwise)
    {
        double sum = 0;
        size_t len = pts.size();
        for (size_t i = 0, j = len > 0 ? len - 1 : 0; i < len; j = i++)
            sum += (pts[j][0] - pts[i][0]) * (pts[i][1] + pts[j][1]);
        int last = -1;
        if (clockwise == (sum > 0)) {
            for (size_t i = 0; i < len; ++i)
                last = insertNode(vertices + (int64_t)i, pts[i][0], pts[i][1], last);
        } else {
            for (size_t i = len; i-- > 0;)
                last = insertNode(vertices + (int64_t)i, pts[i][0], pts[i][1], last);
        }
        if (last >= 0 && equals(last, N(last).next)) {
            removeNode(last);
            last = N(last).next;
        }
        vertices += (int64_t)len;
        return last;
    }

    double area(int p, int q, int r)
    {
        double v = (N(q).y - N(p).y) * (N(r).x - N(q).x) - (N(q).x - N(p).x) * (N(r).y - N(q).y);
        if (std::abs(v) <= std::numeric_limits<double>::epsilon())
            v = 0.0;
        return v;
    }
    bool equals(int a, int b) { return N(a).x == N(b).x && N(a).y == N(b).y; }
    static int sign(double v) { return (0.0 < v) - (v < 0.0); }
    static bool pointInTriangle(double ax, double ay, double bx, double by, double cx, double cy, double px,
                                double py)
    {
        return (cx - px) * (ay - py) - (ax - px) * (cy - py) >= 0 &&
               (ax - px) * (by - py) - (bx - px) * (ay - py) >= 0 &&
               (bx - px) * (cy - py) - (cx - px) * (by - py) >= 0;
    }
    bool onSegment(int p, int q, int r)
    {
        return N(q).x <= std::max(N(p).x, N(r).x) && N(q).x >= std::min(N(p).x, N(r).x) &&
               N(q).y <= std::max(N(p).y, N(r).y) && N(q).y >= std::min(N(p).y, N(r).y);
    }
    bool intersects(int p1, int q1, int p2, int q2)
    {
        int o1 = sign(area(p1, q1, p2));
        int o2 = sign(area(p1, q1, q2));
        int o3 = sign(area(p2, q2, p1));
        int o4 = sign(area(p2, q2, q1));
        if (o1 != o2 && o3 != o4)
            return true;
        if (o1 == 0 && onSegment(p1, p2, q1))
            return true;
        if (o2 == 0 && onSegment(p1, q2, q1))
            return true;
        if (o3 == 0 && onSegment(p2, p1, q2))
            return true;
        if (o4 == 0 && onSegment(p2, q1, q2))
            return true;
        return false;
    }
    bool intersectsPolygon(int a, int b)
    {
        int p = a;
        do {
            int pn = N(p).next;
            if (N(p).i != N(a).i && N(pn).i != N(a).i && N(p).i != N(b).i && N(pn).i != N(b).i &&
                intersects(p, pn, a, b))
                return true;
            p = pn;
        } while (p != a);
        return false;
    }
    bool locallyInside(int a, int b)
    {
        return area(N(a).prev, a, N(a).next) < 0 ? area(a, b, N(a).next) >= 0 && area(a, N(a).prev, b) >= 0
                                                 : area(a, b, N(a).prev) < 0 || area(a, N(a).next, b) < 0;
    }
    bool middleInside(int a, int b)
    {
        int p = a;
        bool inside = false;
        double px = (N(a).x + N(b).x) / 2;
        double py = (N(a).y + N(b).y) / 2;
        do {
            int pn = N(p).next;
            if (((N(p).y > py) != (N(pn).y > py)) && N(pn).y != N(p).y &&
                (px < (N(pn).x - N(p).x) * (py - N(p).y) / (N(pn).y - N(p).y) + N(p).x))
                inside = !inside;
            p = pn;
        } while (p != a);
        return inside;
    }
    bool isValidDiagonal(int a, int b)
    {
        return N(N(a).next).i != N(b).i && N(N(a).prev).i != N(b).i && !intersectsPolygon(a, b) &&
               ((locallyInside(a, b) && locallyInside(b, a) && middleInside(a, b) &&
                 (area(N(a).prev, a, N(b).prev) != 0.0 || area(a, N(b).prev, b) != 0.0)) ||
                (equals(a, b) && area(N(a).prev, a, N(a).next) > 0 && area(N(b).prev, b, N(b).next) > 0));
    }
    int splitPolygon(int a, int b)
    {
        int a2 = newNode(N(a).i, N(a).x, N(a).y);
        int b2 = newNode(N(b).i, N(b).x, N(b).y);
        int an = N(a).next;
        int bp = N(b).prev;
        N(a).next = b;
        N(b).prev = a;
        N(a2).next = an;
        N(an).prev = a2;
        N(b2).next = a2;
        N(a2).prev = b2;
        N(bp).next = b2;
        N(b2).prev = bp;
        return b2;
    }

    int filterPoints(int start, int end = -1)
    {
        if (end < 0)
            end = start;
        int p = start;
        bool again;
        do {
            again = false;
            if (!N(p).steiner && (equals(p, N(p).next) || area(N(p).prev, p, N(p).next) == 0)) {
                removeNode(p);
                p = end = N(p).prev;
                if (p == N(p).next)
                    break;
                again = true;
            } else {
                p = N(p).next;
            }
        } while (again || p != end);
        return end;
    }

    int32_t zOrder(double xd, double yd)
    {
        int32_t x = static_cast<int32_t>(32767.0 * (xd - minX) * invSize);
        int32_t y = static_cast<int32_t>(32767.0 * (yd - minY) * invSize);
        x = (x | (x << 8)) & 0x00FF00FF;
        x = (x | (x << 4)) & 0x0F0F0F0F;
        x = (x | (x << 2)) & 0x33333333;
        x = (x | (x << 1)) & 0x55555555;
        y = (y | (y << 8)) & 0x00FF00FF;
        y = (y | (y << 4)) & 0x0F0F0F0F;
        y = (y | (y << 2)) & 0x33333333;
        y = (y | (y << 1)) & 0x55555555;
        return x | (y << 1);
    }

    void sortLinked(int list)
    {
        int inSize = 1;
        for (;;) {
            int p = list;
            list = -1;
            int tail = -1;
            int numMerges = 0;
            while (p >= 0) {
                numMerges++;
                int q = p;
                int pSize = 0;
                for (int i = 0; i < inSize; i++) {
                    pSize++;
                    q = N(q).nextZ;
                    if (q < 0)
                        break;
                }
                int qSize = inSize;
                while (pSize > 0 || (qSize > 0 && q >= 0)) {
                    int e;
                    if (pSize == 0) {
                        e = q;
                        q = N(q).nextZ;
                        qSize--;
                    } else if (qSize == 0 || q < 0) {
                        e = p;
                        p = N(p).nextZ;
                        pSize--;
                    } else if (N(p).z <= N(q).z) {
                        e = p;
                        p = N(p).nextZ;
                        pSize--;
                    } else {
                        e = q;
                        q = N(q).nextZ;
                        qSize--;
                    }
                    if (tail >= 0)
                        N(tail).nextZ = e;
                    else
                        list = e;
                    N(e).prevZ = tail;
                    tail = e;
                }
                p = q;
            }
            N(tail).nextZ = -1;
            if (numMerges <= 1)
                return;
            inSize *= 2;
        }
    }

    void indexCurve(int start)
    {
        int p = start;
        do {
            N(p).z = N(p).z ? N(p).z : zOrder(N(p).x, N(p).y);
            N(p).prevZ = N(p).prev;
            N(p).nextZ = N(p).next;
            p = N(p).next;
        } while (p != start);
        N(N(p).prevZ).nextZ = -1;
        N(p).prevZ = -1;
        sortLinked(p);
    }

    bool isEar(int ear)
    {
        int a = N(ear).prev, b = ear, c = N(ear).next;
        if (area(a, b, c) >= 0)
            return false;
        int p = N(N(ear).next).next;
        while (p != N(ear).prev) {
            if (pointInTriangle(N(a).x, N(a).y, N(b).x, N(b).y, N(c).x, N(c).y, N(p).x, N(p).y) &&
                area(N(p).prev, p, N(p).next) >= 0)
                return false;
            p = N(p).next;
        }
        return true;
    }

    bool isEarHashed(int ear)
    {
        int a = N(ear).prev, b = ear, c = N(ear).next;
        if (area(a, b, c) >= 0)
            return false;
        double minTX = std::min(N(a).x, std::min(N(b).x, N(c).x));
        double minTY = std::min(N(a).y, std::min(N(b).y, N(c).y));
        double maxTX = std::max(N(a).x, std::max(N(b).x, N(c).x));
        double maxTY = std::max(N(a).y, std::max(N(b).y, N(c).y));
        int32_t minZ = zOrder(minTX, minTY);
        int32_t maxZ = zOrder(maxTX, maxTY);
        int p = N(ear).nextZ;
        while (p >= 0 && N(p).z <= maxZ) {
            if (p != N(ear).prev && p != N(ear).next &&
                pointInTriangle(N(a).x, N(a).y, N(b).x, N(b).y, N(c).x, N(c).y, N(p).x, N(p).y) &&
                area(N(p).prev, p, N(p).next) >= 0)
                return false;
            p = N(p).nextZ;
        }
        p = N(ear).prevZ;
        while (p >= 0 && N(p).z >= minZ) {
            if (p != N(ear).prev && p != N(ear).next &&
                pointInTriangle(N(a).x, N(a).y, N(b).x, N(b).y, N(c).x, N(c).y, N(p).x, N(p).y) &&
                area(N(p).prev, p, N(p).next) >= 0)
                return false;
            p = N(p).prevZ;
        }
        return true;
    }

    int cureLocalIntersections(int start)
    {
        int p = start;
        do {
            int a = N(p).prev;
            int b = N(N(p).next).next;
            if (!equals(a, b) && intersects(a, p, N(p).next, b) && locallyInside(a, b) && locallyInside(b, a)) {
                indices.push_back(N(a).i);
                indices.push_back(N(p).i);
                indices.push_back(N(b).i);
                removeNode(p);
                removeNode(N(p).next);
                p = start = b;
            }
            p = N(p).next;
        } while (p != start);
        return filterPoints(p);
    }

    void splitEarcut(int start)
    {
        int a = start;
        do {
            int b = N(N(a).next).next;
            while (b != N(a).prev) {
                if (N(a).i != N(b).i && isValidDiagonal(a, b)) {
                    int c = splitPolygon(a, b);
                    a = filterPoints(a, N(a).next);
                    c = filterPoints(c, N(c).next);
                    earcutLinked(a, 0);
                    earcutLinked(c, 0);
                    return;
                }
                b = N(b).next;
            }
            a = N(a).next;
        } while (a != start);
    }

    void earcutLinked(int ear, int pass)
    {
        if (ear < 0)
            return;
        if (!pass && hashing)
            indexCurve(ear);
        int stop = ear;
        while (N(ear).prev != N(ear).next) {
            int prev = N(ear).prev;
            int next = N(ear).next;
            if (hashing ? isEarHashed(ear) : isEar(ear)) {
                indices.push_back(N(prev).i);
                indices.push_back(N(ear).i);
                indices.push_back(N(next).i);
                removeNode(ear);
                ear = N(next).next;
                stop = N(next).next;
                continue;
            }
            ear = next;
            if (ear == stop) {
                if (!pass)
                    earcutLinked(filterPoints(ear), 1);
                else if (pass == 1) {
                    ear = cureLocalIntersections(filterPoints(ear));
                    earcutLinked(ear, 2);
                } else if (pass == 2)
                    splitEarcut(ear);
                break;
            }
        }
    }

    int getLeftmost(int start)
    {
        int p = start, left = start;
        do {
            if (N(p).x < N(left).x || (N(p).x == N(left).x && N(p).y < N(left).y))
                left = p;
            p = N(p).next;
        } while (p != start);
        return left;
    }

    bool sectorContainsSector(int m, int p)
    {
        return area(N(m).prev, m, N(p).prev) < 0 && area(N(p).next, m, N(m).next) < 0;
    }

    int findHoleBridge(int hole, int outer)
    {
        int p = outer;
        double hx = N(hole).x, hy = N(hole).y;
        double qx = -std::numeric_limits<double>::infinity();
        int m = -1;
        do {
            int pn = N(p).next;
            if (hy <= N(p).y && hy >= N(pn).y && N(pn).y != N(p).y) {
                double x = N(p).x + (hy - N(p).y) * (N(pn).x - N(p).x) / (N(pn).y - N(p).y);
                if (x <= hx && x > qx) {
                    qx = x;
                    if (x == hx) {
                        if (hy == N(p).y)
                            return p;
                        if (hy == N(pn).y)
                            return pn;
                    }
                    m = N(p).x < N(pn).x ? p : pn;
                }
            }
            p = pn;
        } while (p != outer);
        if (m < 0)
            return -1;
        if (hx == qx)
            return m;
        int stop = m;
        double tanMin = std::numeric_limits<double>::infinity();
        double tanCur = 0;
        p = m;
        double mx = N(m).x, my = N(m).y;
        do {
            if (hx >= N(p).x && N(p).x >= mx && hx != N(p).x &&
                pointInTriangle(hy < my ? hx : qx, hy, mx, my, hy < my ? qx : hx, hy, N(p).x, N(p).y)) {
                tanCur = std::abs(hy - N(p).y) / (hx - N(p).x);
                if (locallyInside(p, hole) &&
                    (tanCur < tanMin || (tanCur == tanMin && (N(p).x > N(m).x || sectorContainsSector(m, p))))) {
                    m = p;
                    tanMin = tanCur;
                }
            }
            p = N(p).next;
        } while (p != stop);
        return m;
    }

    void eliminateHole(int hole, int outer)
    {
        outer = findHoleBridge(hole, outer);
        if (outer >= 0) {
            int b = splitPolygon(outer, hole);
            filterPoints(outer, N(outer).next);
            filterPoints(b, N(b).next);
        }
    }

    int eliminateHoles(const std::vector<std::vector<std::array<double, 2>>> &rings, int outer)
    {
        std::vector<int> queue;
        for (size_t r = 1; r < rings.size(); ++r) {
            int list = linkedList(rings[r], false);
            if (list >= 0) {
                if (list == N(list).next)
                    N(list).steiner = true;
                queue.push_back(getLeftmost(list));
            }
        }
        std::sort(queue.begin(), queue.end(), [this](int a, int b) { return N(a).x < N(b).x; });
        for (size_t k = 0; k < queue.size(); ++k) {
            eliminateHole(queue[k], outer);
            outer = filterPoints(outer, N(outer).next);
        }
        return outer;
    }
};

} // namespace port
