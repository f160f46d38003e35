//! Geometry helpers of `src/common.rs`.
use nalgebra::Vector2;

/// Intersection of segments `line1` and `line2` (`src/common.rs:3-26`):
/// parameters s along `line2` and t along `line1`, both in [0, 1], and the
/// point `p1 + t * (p2 - p1)`.  Parallel segments give a zero denominator, a
/// non-finite s or t, and no intersection.  The f32 operations are the
/// reference's, in its order (the denominator is evaluated twice).
#[inline]
pub fn line_intersection(
    line1: (Vector2<f32>, Vector2<f32>),
    line2: (Vector2<f32>, Vector2<f32>),
) -> Option<Vector2<f32>> {
    let ((p1, p2), (p3, p4)) = (line1, line2);
    let (s1x, s1y) = (p2.x - p1.x, p2.y - p1.y);
    let (s2x, s2y) = (p4.x - p3.x, p4.y - p3.y);
    let s = (-s1y * (p1.x - p3.x) + s1x * (p1.y - p3.y)) / (-s2x * s1y + s1x * s2y);
    let t = (s2x * (p1.y - p3.y) - s2y * (p1.x - p3.x)) / (-s2x * s1y + s1x * s2y);
    if (0.0..=1.0).contains(&s) && (0.0..=1.0).contains(&t) {
        Some(Vector2::new(p1.x + t * s1x, p1.y + t * s1y))
    } else {
        None
    }
}
