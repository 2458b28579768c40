// Device ear-clipping triangulator: the algorithm of the modified mapbox earcut vendored by the reference
// (thirdparty/earcut.hpp/include/mapbox/earcut.hpp) restated over index-linked nodes in caller scratch.
//
// Steps kept identical because the output triangles (not only their union) are compared: winding
// normalisation of each ring (:210-245), collinear/duplicate filtering (:248-271), the three-pass ear loop
// (:274-326) with plain or z-order-hashed ear tests (:329-388, hashing when more than 80 points), local
// self-intersection cure (:391-415), split fallback (:418-442), Eberly hole bridging (:445-544), z-order
// indexing with a linked-list merge sort (:552-658), and area() snapping |value| <= DBL_EPSILON to zero
// (:694-699). The recursion of earcutLinked/splitEarcut is an explicit stack (depth-first, first half
// first, exactly the recursion's order), and every loop carries an iteration budget so a malformed input
// ends with an error instead of spinning.
#pragma once
#include "sb_common.cuh"

namespace sbg {

// std::min / std::max semantics (the second argument wins only when strictly smaller / larger)
SB_HD double smin(double a, double b) { return (b < a) ? b : a; }
SB_HD double smax(double a, double b) { return (a < b) ? b : a; }

struct EcNode {
    double x, y;
    float xf, yf; // round-to-nearest FP32 copies for the filtered orientation tests
    int i;
    int prev, next;
    int z;
    int prevZ, nextZ;
    int steiner;
};

struct DevEarcut {
    EcNode *N = nullptr;
    int cap = 0, cnt = 0;
    int *out = nullptr;
    int outCap = 0, outCnt = 0;
    int2 *stk = nullptr;
    int stkCap = 0, sp = 0;
    int *hq = nullptr; // hole queue
    int vertices = 0;
    bool hashing = false;
    double minX = 0, minY = 0, maxX = 0, maxY = 0, invSize = 0;
    int error = 0; // 1 = capacity, 2 = iteration budget
    long long budget = 0;
    // Filtered orientation tests. Every orientation below is a difference of two products of coordinate
    // differences. Evaluated in FP32 on the FP32 copies, its error against the exact value is at most
    // 48.5 * 2^-24 * M^2 (M: the largest absolute coordinate; input rounding, three roundings per product
    // chain and the final subtraction), and the reference's FP64 evaluation is within 40 * 2^-53 * M^2 of the
    // exact value. So when the FP32 value exceeds 2^-17 M^2 plus a constant that covers the FP64 error (and,
    // for area(), the DBL_EPSILON snap), the FP64 result has the FP32 value's sign and is not snapped; else
    // the FP64 expression is evaluated as the reference does.
    float cmax = 0.f, thrArea = 0x1p-50f, thrOrient = 0x1p-60f;
    bool filtered = true; // false: every orientation in FP64 (the plain FP64 form)

    SB_HD bool tick()
    {
        if (--budget < 0) {
            error = 2;
            return false;
        }
        return true;
    }

    SB_HDF int newNode(int i, double x, double y)
    {
        if (cnt >= cap) {
            error = 1;
            return -1;
        }
        EcNode &n = N[cnt];
        n.x = x;
        n.y = y;
        n.xf = (float)x;
        n.yf = (float)y;
        cmax = fmaxf(cmax, fmaxf(fabsf(n.xf), fabsf(n.yf))); // (a NaN coordinate is skipped: its tests fail
        const float m2 = cmax * cmax;                        //  the filter and fall back to FP64)
        thrArea = filtered ? ldexpf(m2, -17) + 0x1p-50f : INFINITY;
        thrOrient = filtered ? ldexpf(m2, -17) + 0x1p-60f : INFINITY;
        n.i = i;
        n.prev = n.next = -1;
        n.z = 0;
        n.prevZ = n.nextZ = -1;
        n.steiner = 0;
        return cnt++;
    }
    SB_HDF int insertNode(int i, double x, double y, int last)
    {
        int p = newNode(i, x, y);
        if (p < 0)
            return -1;
        if (last < 0) {
            N[p].prev = p;
            N[p].next = p;
        } else {
            N[p].next = N[last].next;
            N[p].prev = last;
            N[N[last].next].prev = p;
            N[last].next = p;
        }
        return p;
    }
    SB_HD void removeNode(int p)
    {
        N[N[p].next].prev = N[p].prev;
        N[N[p].prev].next = N[p].next;
        if (N[p].prevZ >= 0)
            N[N[p].prevZ].nextZ = N[p].nextZ;
        if (N[p].nextZ >= 0)
            N[N[p].nextZ].prevZ = N[p].prevZ;
    }
    SB_HD void emit(int a, int b, int c)
    {
        if (outCnt + 3 > outCap) {
            error = 1;
            return;
        }
        out[outCnt++] = N[a].i;
        out[outCnt++] = N[b].i;
        out[outCnt++] = N[c].i;
    }

    // The reference's area() (:694-699) as far as its callers use it: they compare it with zero only, so a
    // certified FP32 value stands in for the FP64 one (same sign, not snapped).
    SB_HD double area(int p, int q, int r) const
    {
        const float vf = (N[q].yf - N[p].yf) * (N[r].xf - N[q].xf) - (N[q].xf - N[p].xf) * (N[r].yf - N[q].yf);
        if (fabsf(vf) > thrArea)
            return (double)vf;
        double v = (N[q].y - N[p].y) * (N[r].x - N[q].x) - (N[q].x - N[p].x) * (N[r].y - N[q].y);
        if (fabs(v) <= kDblEps)
            v = 0.0;
        return v;
    }
    // one of pointInTriangle's three tests, (c - p) x (a - p) >= 0 in the reference's FP64 form, filtered
    SB_HD bool orientNonNeg(int a, int c, int p) const
    {
        const float ef = (N[c].xf - N[p].xf) * (N[a].yf - N[p].yf) - (N[a].xf - N[p].xf) * (N[c].yf - N[p].yf);
        if (fabsf(ef) > thrOrient)
            return ef > 0.f;
        return (N[c].x - N[p].x) * (N[a].y - N[p].y) - (N[a].x - N[p].x) * (N[c].y - N[p].y) >= 0;
    }
    // pointInTriangle on nodes (the ear tests)
    SB_HD bool nodeInTriangle(int a, int b, int c, int p) const
    {
        return orientNonNeg(a, c, p) && orientNonNeg(b, a, p) && orientNonNeg(c, b, p);
    }
    SB_HD bool equals(int a, int b) const { return N[a].x == N[b].x && N[a].y == N[b].y; }
    static SB_HD int sgn(double v) { return (0.0 < v) - (v < 0.0); }
    static SB_HD bool pointInTriangle(double ax, double ay, double bx, double by, double cx,
                                                           double cy, double px, double py)
    {
        return (cx - px) * (ay - py) - (ax - px) * (cy - py) >= 0 &&
               (ax - px) * (by - py) - (bx - px) * (ay - py) >= 0 &&
               (bx - px) * (cy - py) - (cx - px) * (by - py) >= 0;
    }
    SB_HD bool onSegment(int p, int q, int r) const
    {
        return N[q].x <= smax(N[p].x, N[r].x) && N[q].x >= smin(N[p].x, N[r].x) && N[q].y <= smax(N[p].y, N[r].y) &&
               N[q].y >= smin(N[p].y, N[r].y);
    }
    SB_HDF bool intersects(int p1, int q1, int p2, int q2) const
    {
        int o1 = sgn(area(p1, q1, p2));
        int o2 = sgn(area(p1, q1, q2));
        int o3 = sgn(area(p2, q2, p1));
        int o4 = sgn(area(p2, q2, q1));
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
    SB_HDF bool intersectsPolygon(int a, int b)
    {
        int p = a;
        do {
            int pn = N[p].next;
            if (N[p].i != N[a].i && N[pn].i != N[a].i && N[p].i != N[b].i && N[pn].i != N[b].i &&
                intersects(p, pn, a, b))
                return true;
            p = pn;
        } while (p != a && tick());
        return false;
    }
    SB_HDF bool locallyInside(int a, int b) const
    {
        return area(N[a].prev, a, N[a].next) < 0 ? area(a, b, N[a].next) >= 0 && area(a, N[a].prev, b) >= 0
                                                 : area(a, b, N[a].prev) < 0 || area(a, N[a].next, b) < 0;
    }
    SB_HDF bool middleInside(int a, int b)
    {
        int p = a;
        bool inside = false;
        double px = (N[a].x + N[b].x) / 2;
        double py = (N[a].y + N[b].y) / 2;
        do {
            int pn = N[p].next;
            if (((N[p].y > py) != (N[pn].y > py)) && N[pn].y != N[p].y &&
                (px < (N[pn].x - N[p].x) * (py - N[p].y) / (N[pn].y - N[p].y) + N[p].x))
                inside = !inside;
            p = pn;
        } while (p != a && tick());
        return inside;
    }
    SB_HDF bool isValidDiagonal(int a, int b)
    {
        return N[N[a].next].i != N[b].i && N[N[a].prev].i != N[b].i && !intersectsPolygon(a, b) &&
               ((locallyInside(a, b) && locallyInside(b, a) && middleInside(a, b) &&
                 (area(N[a].prev, a, N[b].prev) != 0.0 || area(a, N[b].prev, b) != 0.0)) ||
                (equals(a, b) && area(N[a].prev, a, N[a].next) > 0 && area(N[b].prev, b, N[b].next) > 0));
    }
    SB_HDF int splitPolygon(int a, int b)
    {
        int a2 = newNode(N[a].i, N[a].x, N[a].y);
        int b2 = newNode(N[b].i, N[b].x, N[b].y);
        if (a2 < 0 || b2 < 0)
            return -1;
        int an = N[a].next;
        int bp = N[b].prev;
        N[a].next = b;
        N[b].prev = a;
        N[a2].next = an;
        N[an].prev = a2;
        N[b2].next = a2;
        N[a2].prev = b2;
        N[bp].next = b2;
        N[b2].prev = bp;
        return b2;
    }
    SB_HDF int filterPoints(int start, int end = -1)
    {
        if (end < 0)
            end = start;
        int p = start;
        bool again;
        do {
            again = false;
            if (!N[p].steiner && (equals(p, N[p].next) || area(N[p].prev, p, N[p].next) == 0)) {
                removeNode(p);
                p = end = N[p].prev;
                if (p == N[p].next)
                    break;
                again = true;
            } else {
                p = N[p].next;
            }
        } while ((again || p != end) && tick());
        return end;
    }
    SB_HDF int zOrder(double xd, double yd) const
    {
        int x = (int)(32767.0 * (xd - minX) * invSize);
        int y = (int)(32767.0 * (yd - minY) * invSize);
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
    SB_HDF void sortLinked(int list)
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
                    q = N[q].nextZ;
                    if (q < 0)
                        break;
                }
                int qSize = inSize;
                while (pSize > 0 || (qSize > 0 && q >= 0)) {
                    int e;
                    if (pSize == 0) {
                        e = q;
                        q = N[q].nextZ;
                        qSize--;
                    } else if (qSize == 0 || q < 0) {
                        e = p;
                        p = N[p].nextZ;
                        pSize--;
                    } else if (N[p].z <= N[q].z) {
                        e = p;
                        p = N[p].nextZ;
                        pSize--;
                    } else {
                        e = q;
                        q = N[q].nextZ;
                        qSize--;
                    }
                    if (tail >= 0)
                        N[tail].nextZ = e;
                    else
                        list = e;
                    N[e].prevZ = tail;
                    tail = e;
                }
                p = q;
                if (!tick())
                    return;
            }
            N[tail].nextZ = -1;
            if (numMerges <= 1)
                return;
            inSize *= 2;
        }
    }
    SB_HDF void indexCurve(int start)
    {
        int p = start;
        do {
            N[p].z = N[p].z ? N[p].z : zOrder(N[p].x, N[p].y);
            N[p].prevZ = N[p].prev;
            N[p].nextZ = N[p].next;
            p = N[p].next;
        } while (p != start && tick());
        N[N[p].prevZ].nextZ = -1;
        N[p].prevZ = -1;
        sortLinked(p);
    }
    SB_HDF bool isEar(int ear)
    {
        int a = N[ear].prev, b = ear, c = N[ear].next;
        if (area(a, b, c) >= 0)
            return false;
        int p = N[N[ear].next].next;
        while (p != N[ear].prev && tick()) {
            if (nodeInTriangle(a, b, c, p) &&
                area(N[p].prev, p, N[p].next) >= 0)
                return false;
            p = N[p].next;
        }
        return true;
    }
    SB_HDF bool isEarHashed(int ear)
    {
        int a = N[ear].prev, b = ear, c = N[ear].next;
        if (area(a, b, c) >= 0)
            return false;
        double minTX = smin(N[a].x, smin(N[b].x, N[c].x));
        double minTY = smin(N[a].y, smin(N[b].y, N[c].y));
        double maxTX = smax(N[a].x, smax(N[b].x, N[c].x));
        double maxTY = smax(N[a].y, smax(N[b].y, N[c].y));
        int minZ = zOrder(minTX, minTY);
        int maxZ = zOrder(maxTX, maxTY);
        int p = N[ear].nextZ;
        while (p >= 0 && N[p].z <= maxZ && tick()) {
            if (p != N[ear].prev && p != N[ear].next &&
                nodeInTriangle(a, b, c, p) &&
                area(N[p].prev, p, N[p].next) >= 0)
                return false;
            p = N[p].nextZ;
        }
        p = N[ear].prevZ;
        while (p >= 0 && N[p].z >= minZ && tick()) {
            if (p != N[ear].prev && p != N[ear].next &&
                nodeInTriangle(a, b, c, p) &&
                area(N[p].prev, p, N[p].next) >= 0)
                return false;
            p = N[p].prevZ;
        }
        return true;
    }
    SB_HDF int cureLocalIntersections(int start)
    {
        int p = start;
        do {
            int a = N[p].prev;
            int b = N[N[p].next].next;
            if (!equals(a, b) && intersects(a, p, N[p].next, b) && locallyInside(a, b) && locallyInside(b, a)) {
                emit(a, p, b);
                removeNode(p);
                removeNode(N[p].next);
                p = start = b;
            }
            p = N[p].next;
        } while (p != start && tick());
        return filterPoints(p);
    }
    // returns true when a split was made (the two halves are pushed on the work stack)
    SB_HDF bool splitEarcut(int start)
    {
        int a = start;
        do {
            int b = N[N[a].next].next;
            while (b != N[a].prev && tick()) {
                if (N[a].i != N[b].i && isValidDiagonal(a, b)) {
                    int c = splitPolygon(a, b);
                    if (c < 0)
                        return false;
                    a = filterPoints(a, N[a].next);
                    c = filterPoints(c, N[c].next);
                    if (sp + 2 > stkCap) {
                        error = 1;
                        return false;
                    }
                    stk[sp++] = make_int2(c, 0); // runs second
                    stk[sp++] = make_int2(a, 0); // runs first
                    return true;
                }
                b = N[b].next;
            }
            a = N[a].next;
        } while (a != start && tick());
        return false;
    }
    // earcutLinked with its recursion unrolled onto the work stack
    SB_HDF void earcutLinked(int ear0, int pass0)
    {
        sp = 0;
        stk[sp++] = make_int2(ear0, pass0);
        while (sp > 0 && !error) {
            int2 job = stk[--sp];
            int ear = job.x, pass = job.y;
            bool restart = true;
            while (restart && !error) {
                restart = false;
                if (ear < 0)
                    break;
                if (!pass && hashing)
                    indexCurve(ear);
                int stop = ear;
                while (N[ear].prev != N[ear].next && tick()) {
                    int prev = N[ear].prev;
                    int next = N[ear].next;
                    if (hashing ? isEarHashed(ear) : isEar(ear)) {
                        emit(prev, ear, next);
                        removeNode(ear);
                        ear = N[next].next;
                        stop = N[next].next;
                        continue;
                    }
                    ear = next;
                    if (ear == stop) {
                        if (!pass) {
                            ear = filterPoints(ear);
                            pass = 1;
                            restart = true;
                        } else if (pass == 1) {
                            ear = cureLocalIntersections(filterPoints(ear));
                            pass = 2;
                            restart = true;
                        } else if (pass == 2) {
                            splitEarcut(ear);
                        }
                        break;
                    }
                }
            }
        }
    }
    SB_HDF int getLeftmost(int start)
    {
        int p = start, left = start;
        do {
            if (N[p].x < N[left].x || (N[p].x == N[left].x && N[p].y < N[left].y))
                left = p;
            p = N[p].next;
        } while (p != start && tick());
        return left;
    }
    SB_HDF bool sectorContainsSector(int m, int p) const
    {
        return area(N[m].prev, m, N[p].prev) < 0 && area(N[p].next, m, N[m].next) < 0;
    }
    SB_HDF int findHoleBridge(int hole, int outer)
    {
        int p = outer;
        double hx = N[hole].x, hy = N[hole].y;
        double qx = -(double)INFINITY;
        int m = -1;
        do {
            int pn = N[p].next;
            if (hy <= N[p].y && hy >= N[pn].y && N[pn].y != N[p].y) {
                double x = N[p].x + (hy - N[p].y) * (N[pn].x - N[p].x) / (N[pn].y - N[p].y);
                if (x <= hx && x > qx) {
                    qx = x;
                    if (x == hx) {
                        if (hy == N[p].y)
                            return p;
                        if (hy == N[pn].y)
                            return pn;
                    }
                    m = N[p].x < N[pn].x ? p : pn;
                }
            }
            p = pn;
        } while (p != outer && tick());
        if (m < 0)
            return -1;
        if (hx == qx)
            return m;
        int stop = m;
        double tanMin = (double)INFINITY;
        double tanCur = 0;
        p = m;
        double mx = N[m].x, my = N[m].y;
        do {
            if (hx >= N[p].x && N[p].x >= mx && hx != N[p].x &&
                pointInTriangle(hy < my ? hx : qx, hy, mx, my, hy < my ? qx : hx, hy, N[p].x, N[p].y)) {
                tanCur = fabs(hy - N[p].y) / (hx - N[p].x);
                if (locallyInside(p, hole) &&
                    (tanCur < tanMin || (tanCur == tanMin && (N[p].x > N[m].x || sectorContainsSector(m, p))))) {
                    m = p;
                    tanMin = tanCur;
                }
            }
            p = N[p].next;
        } while (p != stop && tick());
        return m;
    }
    SB_HDF void eliminateHole(int hole, int outer)
    {
        outer = findHoleBridge(hole, outer);
        if (outer >= 0) {
            int b = splitPolygon(outer, hole);
            if (b < 0)
                return;
            filterPoints(outer, N[outer].next);
            filterPoints(b, N[b].next);
        }
    }
    // ring: coordinates pts2[ids[k]] for k in [0, len); returns the last inserted node or -1
    SB_HDF int linkedList(const d2 *pts2, const int *ids, int len, bool clockwise)
    {
        double sum = 0;
        for (int i = 0, j = len > 0 ? len - 1 : 0; i < len; j = i++)
            sum += (pts2[ids[j]].x - pts2[ids[i]].x) * (pts2[ids[i]].y + pts2[ids[j]].y);
        int last = -1;
        if (clockwise == (sum > 0)) {
            for (int i = 0; i < len; ++i)
                last = insertNode(vertices + i, pts2[ids[i]].x, pts2[ids[i]].y, last);
        } else {
            for (int i = len - 1; i >= 0; --i)
                last = insertNode(vertices + i, pts2[ids[i]].x, pts2[ids[i]].y, last);
        }
        if (error)
            return -1;
        if (last >= 0 && equals(last, N[last].next)) {
            removeNode(last);
            last = N[last].next;
        }
        vertices += len;
        return last;
    }

    // rings: ring r is ids[off[r] .. off[r+1]); output indices are flattened positions (into ids)
    SB_HDF void run(const d2 *pts2, const int *ids, const int *off, int nrings)
    {
        outCnt = 0;
        cnt = 0;
        vertices = 0;
        if (nrings <= 0)
            return;
        int threshold = 80;
        for (int r = 0; threshold >= 0 && r < nrings; ++r)
            threshold -= off[r + 1] - off[r];
        int outer = linkedList(pts2, ids + off[0], off[1] - off[0], true);
        if (outer < 0 || N[outer].prev == N[outer].next)
            return;
        if (nrings > 1) {
            int nq = 0;
            for (int r = 1; r < nrings; ++r) {
                int list = linkedList(pts2, ids + off[r], off[r + 1] - off[r], false);
                if (error)
                    return;
                if (list >= 0) {
                    if (list == N[list].next)
                        N[list].steiner = 1;
                    hq[nq++] = getLeftmost(list);
                }
            }
            // sort by x; a stable insertion sort equals the library sort for up to 16 holes
            for (int k = 1; k < nq; ++k) {
                int v = hq[k];
                int j = k - 1;
                while (j >= 0 && N[v].x < N[hq[j]].x) {
                    hq[j + 1] = hq[j];
                    --j;
                }
                hq[j + 1] = v;
            }
            for (int k = 0; k < nq && !error; ++k) {
                eliminateHole(hq[k], outer);
                outer = filterPoints(outer, N[outer].next);
            }
        }
        hashing = threshold < 0;
        if (hashing) {
            int p = N[outer].next;
            minX = maxX = N[outer].x;
            minY = maxY = N[outer].y;
            do {
                double x = N[p].x, y = N[p].y;
                minX = smin(minX, x);
                minY = smin(minY, y);
                maxX = smax(maxX, x);
                maxY = smax(maxY, y);
                p = N[p].next;
            } while (p != outer && tick());
            invSize = smax(maxX - minX, maxY - minY);
            invSize = invSize != 0.0 ? (1.0 / invSize) : 0.0;
        }
        earcutLinked(outer, 0);
    }
};

} // namespace sbg
