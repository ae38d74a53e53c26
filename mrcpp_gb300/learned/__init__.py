"""Learned output grid: training and evaluation of the grid network."""
