"""Stand-in for scikit-image (absent here) used only when the golden fixtures
are generated: it lets the reference's Utils module import, and records what
the reference passes to skimage.transform.resize (test infrastructure)."""
