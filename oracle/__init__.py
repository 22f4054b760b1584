"""CPU oracle of the raytracer_3D time-stepping path (test infrastructure only)."""
