"""bmnd_gb300 package (placeholder while the API is being laid down)."""
